/*
 * CPU restatement of the SimFast21 HII-bubble stage.  TEST INFRASTRUCTURE:
 * the parity checker and the timed CPU baseline; never part of the product.
 *
 * Every step restates the reference file:line it follows; the floating
 * point operation order is the reference's (C99, no FMA contraction), so
 * with the same FFT implementation the result is byte-identical.
 */
#define _POSIX_C_SOURCE 200809L
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fftw3.h"
#include "hii_oracle.h"

#define ORA_CM_PER_MPC 3.0857e24 /* get_HIIbubbles.c:30, user_functions.c:26 */
#define ORA_V_NORM 1.e+45        /* user_functions.c:38 */

/* ---- user_functions.c:40-47 : ionisation rate of a halo of mass M ------ */
double sf21o_Rion(float hmass, double z, const sf21o_params *p) {
  (void)p;
  const double a1 = 1.575e39, a2 = 9.367608e+07, a3 = 0.44, a4 = 2.27044695e+00;
  double t1 = a1 * hmass * pow((1.0 + z), a4);
  double t2 = pow((hmass / a2), a3);
  double t3 = exp(-pow((a2 / hmass), 3.0));
  double t4 = t1 * t2 * t3;
  return t4 / ORA_V_NORM;
}

/* ---- user_functions.c:58-65 : recombination rate for overdensity 1+d --- */
double sf21o_Rrec(float overdensity, double z, const sf21o_params *p) {
  const double b1 = 9.84815696, b2 = 1.76105133, b3 = 0.81722878,
               b4 = 5.06773134;
  double q1 = 1.e-24 * b1 * pow((1.0 + z), b4);
  double q2 = pow((overdensity / b2), b3);
  double q3 = pow(q2 / (1. + q2), 4.);
  double cell = pow(p->L * ORA_CM_PER_MPC / p->N / p->hubble / (1. + z), 3.0);
  return q1 * q3 * cell / ORA_V_NORM;
}

/* ---- user_functions.c:84-88 -------------------------------------------- */
double sf21o_Qion(double z) {
  return pow(10.0, 2.05707274e-02 * z + 5.29944413e+01) / ORA_V_NORM;
}

/* ---- user_functions.c:92-97 -------------------------------------------- */
double sf21o_G_H(double z) {
  double lo = -4.37152818e-05 * pow(z, 5.) + 1.64394635e-03 * pow(z, 4.) -
              2.03044756e-02 * pow(z, 3.);
  double hi = 7.18335221e-02 * pow(z, 2.) - 8.85791388e-02 * z - 1.20887500e+01;
  return 4.19232273531e-13 / pow(10.0, lo + hi);
}

/* ---- user_functions.c:101-106 : residual neutral fraction -------------- */
double sf21o_XHI(double r) {
  double num = 2. * r + 1. - sqrt((2. * r + 1.) * (2. * r + 1.) - 4. * r * r);
  double val = num / (2. * r);
  if (r == 0.0) return 0.0;
  return val;
}

/* ---- auxiliary.c:350-359 : real-space top-hat window in k-space -------- */
double sf21o_W_filter(double x) {
  double j1onx;
  if (x < 0.03)
    j1onx = (1.0 / 3.0 - x * x * 1.0 / 30.0);
  else
    j1onx = -(cos(x) - (sin(x) / x)) / x / x;
  return 3.0 * j1onx;
}

/* ---- auxiliary.c:537-544 ------------------------------------------------ */
static long wrap_index(long x, long n) {
  x = x % n;
  if (x < 0) x += n;
  return x;
}

/* ---- Input_variables.c:128-129 and get_HIIbubbles.c:192 ---------------- */
static double cell_size(const sf21o_params *p) { return p->L / p->N; }
static double radius_ratio(const sf21o_params *p) {
  return pow(10.0, log10(p->Rmax / cell_size(p)) / p->Nbins);
}

int sf21o_radii(const sf21o_params *p, double *R, int cap, int *n_fft) {
  const double dx = cell_size(p), b = radius_ratio(p);
  double r = p->Rmax;
  int n = 0, nf = 0;
  while (r >= 2 * dx) { /* :299 */
    if (n < cap) R[n] = r;
    n++; nf++;
    r /= b; /* :397 */
  }
  while (r >= dx) { /* :402 */
    if (n < cap) R[n] = r;
    n++;
    r /= b; /* :461 */
  }
  if (n_fft) *n_fft = nf;
  return n;
}

typedef struct {
  long N, N3, Nh;
  float *rec, *ion, *top, *bub, *fill, *fres;
  fftwf_complex *rec_c, *ion_c, *recf_c, *ionf_c, *top_c, *bub_c;
  fftwf_plan f_rec, f_ion, i_rec, i_ion, f_top, f_bub, i_bub;
} work_t;

static void work_free(work_t *w) {
  fftwf_plan *pl[] = {&w->f_rec, &w->f_ion, &w->i_rec, &w->i_ion,
                      &w->f_top, &w->f_bub, &w->i_bub};
  for (unsigned i = 0; i < sizeof(pl) / sizeof(pl[0]); i++)
    if (*pl[i]) fftwf_destroy_plan(*pl[i]);
  void *bufs[] = {w->rec, w->ion, w->top, w->bub, w->fill, w->fres,
                  w->rec_c, w->ion_c, w->recf_c, w->ionf_c, w->top_c, w->bub_c};
  for (unsigned i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++) fftwf_free(bufs[i]);
}

/* Allocation and plans: get_HIIbubbles.c:98-183. */
static int work_init(work_t *w, const sf21o_params *p) {
  memset(w, 0, sizeof(*w));
  const long N = p->N;
  w->N = N;
  w->N3 = N * N * N;
  w->Nh = N * N * (N / 2 + 1);
  fftwf_plan_with_nthreads(p->nthreads > 0 ? p->nthreads : 1);
  w->rec = fftwf_malloc(sizeof(float) * w->N3);
  w->ion = fftwf_malloc(sizeof(float) * w->N3);
  w->top = fftwf_malloc(sizeof(float) * w->N3);
  w->bub = fftwf_malloc(sizeof(float) * w->N3);
  w->fill = fftwf_malloc(sizeof(float) * w->N3);
  w->fres = fftwf_malloc(sizeof(float) * w->N3);
  w->rec_c = fftwf_malloc(sizeof(fftwf_complex) * w->Nh);
  w->ion_c = fftwf_malloc(sizeof(fftwf_complex) * w->Nh);
  w->recf_c = fftwf_malloc(sizeof(fftwf_complex) * w->Nh);
  w->ionf_c = fftwf_malloc(sizeof(fftwf_complex) * w->Nh);
  w->top_c = fftwf_malloc(sizeof(fftwf_complex) * w->Nh);
  w->bub_c = fftwf_malloc(sizeof(fftwf_complex) * w->Nh);
  if (!w->rec || !w->ion || !w->top || !w->bub || !w->fill || !w->fres ||
      !w->rec_c || !w->ion_c || !w->recf_c || !w->ionf_c || !w->top_c ||
      !w->bub_c) {
    work_free(w);
    return 1;
  }
  const int n = (int)N;
  w->f_rec = fftwf_plan_dft_r2c_3d(n, n, n, w->rec, w->rec_c, FFTW_MEASURE);
  w->f_ion = fftwf_plan_dft_r2c_3d(n, n, n, w->ion, w->ion_c, FFTW_MEASURE);
  w->i_rec = fftwf_plan_dft_c2r_3d(n, n, n, w->recf_c, w->rec, FFTW_MEASURE);
  w->i_ion = fftwf_plan_dft_c2r_3d(n, n, n, w->ionf_c, w->ion, FFTW_MEASURE);
  w->f_top = fftwf_plan_dft_r2c_3d(n, n, n, w->top, w->top_c, FFTW_MEASURE);
  w->f_bub = fftwf_plan_dft_r2c_3d(n, n, n, w->bub, w->bub_c, FFTW_MEASURE);
  w->i_bub = fftwf_plan_dft_c2r_3d(n, n, n, w->bub_c, w->bub, FFTW_MEASURE);
  if (!w->f_rec || !w->f_ion || !w->i_rec || !w->i_ion || !w->f_top ||
      !w->f_bub || !w->i_bub) {
    work_free(w);
    return 1;
  }
  return 0;
}

/* k-space top-hat filter of both spectra at radius R: :305-322 (and the
 * identical loop at :406-423).  float complex * double -> float complex. */
static void filter_spectra(const work_t *w, const sf21o_params *p, double R) {
  const long N = w->N, Nh = N / 2 + 1;
  const double dk = 2 * 3.1415926535897932385E0 / p->L; /* Input_variables.c:127 */
  const float *rc = (const float *)w->rec_c, *ic = (const float *)w->ion_c;
  float *rf = (float *)w->recf_c, *inf = (float *)w->ionf_c;
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
  for (long i = 0; i < N; i++) {
    long ki = i > N / 2 ? -(N - i) : i;
    for (long j = 0; j < N; j++) {
      long kj = j > N / 2 ? -(N - j) : j;
      for (long q = 0; q <= N / 2; q++) {
        double kk = dk * sqrt(ki * ki + kj * kj + q * q);
        long e = 2 * (i * N * Nh + j * Nh + q);
        double wf = sf21o_W_filter(kk * R);
        rf[e] = (float)((double)rc[e] * wf);
        rf[e + 1] = (float)((double)rc[e + 1] * wf);
        double wg = sf21o_W_filter(kk * R);
        inf[e] = (float)((double)ic[e] * wg);
        inf[e + 1] = (float)((double)ic[e + 1] * wg);
      }
    }
  }
}

/* Recombination-rate box, residual neutral fraction, cleared bubble box:
 * get_HIIbubbles.c:216-225. */
static void prologue(work_t *w, const sf21o_params *p, double z,
                     const float *delta) {
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
  for (long i = 0; i < w->N3; i++) {
    float d = delta[i];
    float fr = (float)((1. + d) * 1.881e-7 * pow(1. + z, 3.0) * sf21o_G_H(z));
    w->fres[i] = (float)sf21o_XHI(fr);
    w->rec[i] = (float)sf21o_Rrec((float)(1.0 + d), z, p);
    w->fill[i] = 0.0f;
  }
}

/* Single-cell fill: :281-288. */
static void single_cell_fill(work_t *w, const sf21o_params *p) {
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
  for (long i = 0; i < w->N3; i++) {
    double t;
    if (w->ion[i] > 0.) {
      if (w->rec[i] > 0.)
        t = (double)w->ion[i] / w->rec[i];
      else
        t = 1.0;
    } else
      t = 0.;
    if (t >= 1.0)
      w->fill[i] = 1.0f;
    else
      w->fill[i] = (float)t;
  }
}

/* One radius of the FFT branch (R >= 2 dx, :305-393): filter, both inverse
 * transforms, centre test and, when there are centres, the FP32 convolution
 * with the discrete sphere and its threshold into the fill box. */
static void radius_fft(work_t *w, const sf21o_params *p, double R) {
  const long N = w->N, N3 = w->N3;
  const double dx = cell_size(p);
  const double dx3 = pow(dx, 3);
  filter_spectra(w, p, R);
  fftwf_execute(w->i_rec);
  fftwf_execute(w->i_ion);
  int any = 0;
  /* centre test :335-352 */
#pragma omp parallel for num_threads(p->nthreads) schedule(static) reduction(| : any)
  for (long i = 0; i < N3; i++) {
    float h = w->ion[i], d = w->rec[i];
    float c = 0.0f;
    if (h > 0.) {
      if (d > 0.) {
        if ((double)h / d >= 1.0) c = 1.0f;
      } else
        c = 1.0f;
    }
    w->bub[i] = c;
    if (c != 0.0f) any = 1;
  }
  if (any) {
    /* discrete periodic sphere :363-371 (8 image tests) */
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
    for (long i = 0; i < N; i++)
      for (long j = 0; j < N; j++)
        for (long q = 0; q < N; q++) {
          long im = i - N, jm = j - N, qm = q - N;
          int in =
              sqrt(i * i + j * j + q * q) * dx <= R ||
              sqrt(i * i + jm * jm + q * q) * dx <= R ||
              sqrt(i * i + jm * jm + qm * qm) * dx <= R ||
              sqrt(i * i + qm * qm + j * j) * dx <= R ||
              sqrt(im * im + j * j + q * q) * dx <= R ||
              sqrt(im * im + jm * jm + q * q) * dx <= R ||
              sqrt(im * im + jm * jm + qm * qm) * dx <= R ||
              sqrt(im * im + j * j + qm * qm) * dx <= R;
          w->top[i * N * N + j * N + q] = in ? 1.0f : 0.0f;
        }
    fftwf_execute(w->f_top); /* :372 */
    fftwf_execute(w->f_bub); /* :373 */
    /* complex product :379-381 (float complex *= float complex) */
    float *bc = (float *)w->bub_c;
    const float *tc = (const float *)w->top_c;
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
    for (long i = 0; i < w->Nh; i++) {
      float a = bc[2 * i], b = bc[2 * i + 1], c = tc[2 * i], d = tc[2 * i + 1];
      float ac = a * c, bd = b * d, ad = a * d, bcv = b * c;
      bc[2 * i] = ac - bd;
      bc[2 * i + 1] = ad + bcv;
    }
    fftwf_execute(w->i_bub); /* :382 */
    /* threshold :390-393 */
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
    for (long i = 0; i < N3; i++) {
      w->bub[i] = (float)((double)w->bub[i] * dx3 / (double)N3);
      if ((double)w->bub[i] > dx3 / 100) w->fill[i] = 1.0f;
    }
  }
}

/* One radius of the small-R branch (dx <= R < 2 dx, :406-458): filter, both
 * inverse transforms and the painting of each centre's ball. */
static void radius_small(work_t *w, const sf21o_params *p, double R) {
  const long N = w->N;
  const double dx = cell_size(p);
  filter_spectra(w, p, R);
  fftwf_execute(w->i_rec);
  fftwf_execute(w->i_ion);
  const long nc = (long)(R / dx); /* :428 */
  /* painting :433-458; concurrent writers all store 1.0 */
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
  for (long ic = 0; ic < N; ic++)
    for (long jc = 0; jc < N; jc++)
      for (long kc = 0; kc < N; kc++) {
        long c = ic * N * N + jc * N + kc;
        float h = w->ion[c], d = w->rec[c];
        if (!(h > 0.)) continue;
        if (!(!(d > 0.) || ((double)h / d >= 1.0))) continue;
        for (long a = -(nc + 1); a <= nc + 1; a++) {
          long ai = wrap_index(ic + a, N);
          for (long b = -(nc + 1); b <= nc + 1; b++) {
            if (!(sqrt(a * a + b * b) * dx <= R)) continue;
            long bi = wrap_index(jc + b, N);
            for (long e = -(nc + 1); e <= nc + 1; e++) {
              long ei = wrap_index(kc + e, N);
              if (sqrt(a * a + b * b + e * e) * dx <= R)
                w->fill[ai * N * N + bi * N + ei] = 1.0f;
            }
          }
        }
      }
}

/* Radius loops (:298-462), cap (:466-471), neutral fraction (:473-477). */
static void bubble_loops(work_t *w, const sf21o_params *p, float *xhii,
                         double *neutral) {
  const long N3 = w->N3;
  const double dx = cell_size(p), bf = radius_ratio(p);
  double R = p->Rmax;

  int done = 0;
  const int cap = p->max_radii > 0 ? p->max_radii : 1 << 30;

  fftwf_execute(w->f_rec); /* :290 */
  fftwf_execute(w->f_ion); /* :291 */

  while (R >= 2 * dx && done++ < cap) {
    radius_fft(w, p, R);
    R /= bf;
  }

  while (R >= dx && done++ < cap) {
    radius_small(w, p, R);
    R /= bf;
  }

  /* cap :469-471 */
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
  for (long i = 0; i < N3; i++)
    if (w->fill[i] > 1.0 - w->fres[i]) w->fill[i] = 1.0 - w->fres[i];

  /* neutral fraction :473-477 (serial double sum, reference order) */
  double nsum = 0.;
  for (long i = 0; i < N3; i++) nsum += 1.0 - w->fill[i];
  nsum /= N3;
  if (neutral) *neutral = nsum;
  memcpy(xhii, w->fill, sizeof(float) * N3);
}

static int run_common(const sf21o_params *p, double z, const float *delta,
                      const float *src, int src_is_sfrd, float *xhii,
                      float *fresid, float *rec0, float *ion0, float *fill0,
                      double *neutral) {
  work_t w;
  if (work_init(&w, p)) return 1;
  prologue(&w, p, z, delta);
  const double dx = cell_size(p);
  if (src_is_sfrd) {
    /* SFRD -> Rion : :272-274 */
    const double q = sf21o_Qion(z);
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
    for (long i = 0; i < w.N3; i++)
      w.ion[i] = (float)(src[i] * dx * dx * dx * q * p->fesc);
  } else {
    memcpy(w.ion, src, sizeof(float) * w.N3);
  }
  single_cell_fill(&w, p);
  if (fresid) memcpy(fresid, w.fres, sizeof(float) * w.N3);
  if (rec0) memcpy(rec0, w.rec, sizeof(float) * w.N3);
  if (ion0) memcpy(ion0, w.ion, sizeof(float) * w.N3);
  if (fill0) memcpy(fill0, w.fill, sizeof(float) * w.N3);
  if (p->max_radii < 0)
    memcpy(xhii, w.fill, sizeof(float) * w.N3);
  else
    bubble_loops(&w, p, xhii, neutral);
  work_free(&w);
  return 0;
}

/* CPU-baseline timing sample (SFR branch): the front of one redshift --
 * prologue, source conversion, single-cell fill and both forward transforms
 * (:216-291) -- timed once, then the loop body of each listed radius index
 * on its own (a radius's body depends on the others only through the fill
 * box, which it only sets), timed one by one.  Wall times in seconds. */
int sf21o_time_radii(const sf21o_params *p, double z, const float *delta,
                     const float *sfrd, const int *ridx, int n,
                     double *t_front, double *t_radius) {
  double R[512];
  int n_fft = 0;
  const int nr = sf21o_radii(p, R, 512, &n_fft);
  for (int k = 0; k < n; k++)
    if (ridx[k] < 0 || ridx[k] >= nr || nr > 512) return 2;
  work_t w;
  if (work_init(&w, p)) return 1;
  const double t0 = omp_get_wtime();
  prologue(&w, p, z, delta);
  const double dx = cell_size(p);
  const double q = sf21o_Qion(z);
#pragma omp parallel for num_threads(p->nthreads) schedule(static)
  for (long i = 0; i < w.N3; i++)
    w.ion[i] = (float)(sfrd[i] * dx * dx * dx * q * p->fesc);
  single_cell_fill(&w, p);
  fftwf_execute(w.f_rec);
  fftwf_execute(w.f_ion);
  *t_front = omp_get_wtime() - t0;
  for (int k = 0; k < n; k++) {
    const double t1 = omp_get_wtime();
    if (ridx[k] < n_fft)
      radius_fft(&w, p, R[ridx[k]]);
    else
      radius_small(&w, p, R[ridx[k]]);
    t_radius[k] = omp_get_wtime() - t1;
  }
  work_free(&w);
  return 0;
}

int sf21o_run_z_sfr(const sf21o_params *p, double z, const float *delta,
                    const float *sfrd, float *xhii, float *fresid, float *rec0,
                    float *ion0, float *fill0, double *neutral) {
  return run_common(p, z, delta, sfrd, 1, xhii, fresid, rec0, ion0, fill0,
                    neutral);
}

int sf21o_run_z_rion(const sf21o_params *p, double z, const float *delta,
                     const float *rion, float *xhii, float *fresid,
                     float *rec0, float *fill0, double *neutral) {
  return run_common(p, z, delta, rion, 0, xhii, fresid, rec0, NULL, fill0,
                    neutral);
}

/* ---- auxiliary.c:761-808 : cloud-in-cell deposit of one value ---------- */
static void cic_deposit(float x1, float y1, float z1, float val, float *map,
                        long N) {
  long x = (long)x1, y = (long)y1, z = (long)z1;
  x1 -= x;
  y1 -= y;
  z1 -= z;
  for (long a = 0; a < 2; a++)
    for (long b = 0; b < 2; b++)
      for (long c = 0; c < 2; c++) {
        x += a;
        y += b;
        z += c;
        if (x1 < 0.0) { x = x - 1; x1 = fabsf(x1); }
        if (y1 < 0.0) { y = y - 1; y1 = fabsf(y1); }
        if (z1 < 0.0) { z = z - 1; z1 = fabsf(z1); }
        x = wrap_index(x, N);
        y = wrap_index(y, N);
        z = wrap_index(z, N);
        if (a == 1) x1 = 1.0 - x1;
        if (b == 1) y1 = 1.0 - y1;
        if (c == 1) z1 = 1.0 - z1;
        map[x * N * N + y * N + z] += (1.0 - x1) * (1.0 - y1) * (1.0 - z1) * val;
        x -= a;
        y -= b;
        z -= c;
        if (a == 1) x1 = 1.0 - x1;
        if (b == 1) y1 = 1.0 - y1;
        if (c == 1) z1 = 1.0 - z1;
      }
}

/* ---- auxiliary.c:643-684 : block-average N^3 -> Ns^3 -------------------- */
static void block_average(const float *box, float *out, long N, long Ns,
                          int nthreads) {
  long sm = (long)roundf((1.0 * N) / Ns);
  if (Ns * sm > N) sm = sm - 1;
  const double sm3 = 1.0 * sm * sm * sm;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (long i = 0; i < Ns; i++)
    for (long j = 0; j < Ns; j++)
      for (long q = 0; q < Ns; q++) {
        double av = 0.0;
        for (long a = 0; a < sm; a++)
          for (long b = 0; b < sm; b++)
            for (long c = 0; c < sm; c++)
              av += box[(i * sm + a) * N * N + (j * sm + b) * N + (q * sm + c)];
        out[i * Ns * Ns + j * Ns + q] = (float)(av / sm3);
      }
}

int sf21o_halo_source(const sf21o_params *p, double z, long nhalos,
                      const sf21o_halo *halos, float *out) {
  int rc = sf21o_halo_smoothed(p, z, nhalos, halos, out);
  if (rc) return rc;
  const long N = p->N;
  const double dxs = p->L / N, dxh = p->L / p->N_halo;
  const long N3 = N * N * N;
  for (long i = 0; i < N3; i++) /* :257-259 */
    out[i] = out[i] * pow(dxs / dxh, 3) * p->fesc;
  return 0;
}

int sf21o_halo_smoothed(const sf21o_params *p, double z, long nhalos,
                        const sf21o_halo *halos, float *out) {
  const long Nh = p->N_halo, N = p->N;
  if (N > Nh) return 2; /* smooth_box rejects Ns > N (auxiliary.c:651-654) */
  float *fine = calloc((size_t)(Nh * Nh * Nh), sizeof(float));
  if (!fine) return 1;
  for (long i = 0; i < nhalos; i++) /* :249-251, serial */
    cic_deposit(halos[i].x, halos[i].y, halos[i].z,
                sf21o_Rion(halos[i].Mass, z, p), fine, Nh);
  block_average(fine, out, Nh, N, p->nthreads > 0 ? p->nthreads : 1);
  free(fine);
  return 0;
}

/* ---- get_SFR.c:104-146 : SFRD box of one catalogue ---------------------
 * sfr(M, z) = Rion(M, z) / Qion(z) (user_functions.c:71-75) into CIC's float
 * weight on the N_halo^3 grid (:119-121), block average (:123), then each
 * cell / pow(dx_halo, 3) in double, rounded to float (:129-131); mean is the
 * serial double sum / N^3 (:141-145). */
int sf21o_sfrd_box(const sf21o_params *p, double z, long nhalos,
                   const sf21o_halo *halos, float *out, double *mean) {
  const long Nh = p->N_halo, N = p->N;
  if (N > Nh) return 2;
  float *fine = calloc((size_t)(Nh * Nh * Nh), sizeof(float));
  if (!fine) return 1;
  const double q = sf21o_Qion(z);
  for (long i = 0; i < nhalos; i++)
    cic_deposit(halos[i].x, halos[i].y, halos[i].z,
                (float)(sf21o_Rion(halos[i].Mass, z, p) / q), fine, Nh);
  block_average(fine, out, Nh, N, p->nthreads > 0 ? p->nthreads : 1);
  free(fine);
  const double dxh = p->L / Nh;
  const long N3 = N * N * N;
  for (long i = 0; i < N3; i++) out[i] = out[i] / pow(dxh, 3);
  if (mean) {
    double s = 0.0;
    for (long i = 0; i < N3; i++) s += out[i];
    *mean = s / N3;
  }
  return 0;
}

int sf21o_filtered(const sf21o_params *p, const float *rec0, const float *ion0,
                   double R, float *rec_R, float *ion_R) {
  work_t w;
  if (work_init(&w, p)) return 1;
  memcpy(w.rec, rec0, sizeof(float) * w.N3);
  memcpy(w.ion, ion0, sizeof(float) * w.N3);
  fftwf_execute(w.f_rec);
  fftwf_execute(w.f_ion);
  filter_spectra(&w, p, R);
  fftwf_execute(w.i_rec);
  fftwf_execute(w.i_ion);
  memcpy(rec_R, w.rec, sizeof(float) * w.N3);
  memcpy(ion_R, w.ion, sizeof(float) * w.N3);
  work_free(&w);
  return 0;
}
