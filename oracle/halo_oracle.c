/*
 * CPU restatement of SimFast21's excursion-set halo finder, get_halos.c
 * (TEST INFRASTRUCTURE ONLY; see halo_oracle.h).  Same arithmetic in the
 * same order as the reference, so that with the same FFT (the shim) the
 * catalogues are byte-identical.
 */
#include "halo_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"

#define H_PI 3.1415926535897932385E0 /* Input_variables.h:10 */
#define H_RHO0 2.775e11              /* Input_variables.h:11, Msun/h/(Mpc/h)^3 */
#define H_H0 3.24078e-18             /* Input_variables.h:108, h/s */
#define SQ(a) ((a) * (a))

/* ---- Eisenstein & Hu transfer function (auxiliary.c:28-210) ----------------- */
typedef struct {
  double omhh, theta_cmb, growth_k0, alpha_gamma, sound_horizon_fit, beta_c, growth_to_z0;
} eh_parms;

/* the quantities Set_Cosmology (:28-150) leaves for the transfer function */
static void eh_set(const sf21o_hparams *p, double redshift, eh_parms *tf) {
  const double h = p->hubble, omm = p->omega_m, lamb = p->omega_l;
  double omb = p->omega_b;
  const double theta_cmb = 2.728 / 2.7;
  if (omb <= 0) omb = 1e-5;
  const double omega_curv = 1.0 - omm - lamb;
  const double omhh = omm * SQ(h), obhh = omb * SQ(h);
  const double f_baryon = omb / omm, f_cdm = 1.0 - f_baryon;
  const double z_equality = 25000.0 * omhh / SQ(SQ(theta_cmb));
  const double z_drag_b1 = 0.313 * pow(omhh, -0.419) * (1 + 0.607 * pow(omhh, 0.674));
  const double z_drag_b2 = 0.238 * pow(omhh, 0.223);
  const double z_drag =
      1291 * pow(omhh, 0.251) / (1.0 + 0.659 * pow(omhh, 0.828)) * (1.0 + z_drag_b1 * pow(obhh, z_drag_b2));
  const double y_drag = z_equality / (1.0 + z_drag);
  const double sound_horizon_fit = 44.5 * log(9.83 / omhh) / sqrt(1.0 + 10.0 * pow(obhh, 0.75));
  const double p_c = 0.25 * (5.0 - sqrt(1 + 24.0 * f_cdm));
  const double omega_denom = lamb + SQ(1.0 + redshift) * (omega_curv + omm * (1.0 + redshift));
  const double omega_lambda_z = lamb / omega_denom;
  const double omega_matter_z = omm * SQ(1.0 + redshift) * (1.0 + redshift) / omega_denom;
  const double growth_k0 = z_equality / (1.0 + redshift) * 2.5 * omega_matter_z /
                           (pow(omega_matter_z, 4.0 / 7.0) - omega_lambda_z +
                            (1.0 + omega_matter_z / 2.0) * (1.0 + omega_lambda_z / 70.0));
  double growth_to_z0 =
      z_equality * 2.5 * omm / (pow(omm, 4.0 / 7.0) - lamb + (1.0 + omm / 2.0) * (1.0 + lamb / 70.0));
  growth_to_z0 = growth_k0 / growth_to_z0;
  const double alpha_nu = (1 - f_baryon) * (5 - 2 * p_c) / (5) * pow(1 + y_drag, -p_c) *
                          (1 + f_baryon * (-0.553 + 0.126 * f_baryon * f_baryon)) *
                          (1 + (p_c) / 2 * (1 + 1 / (3. - 4. * p_c) / (7.)) / (1 + y_drag));
  tf->omhh = omhh;
  tf->theta_cmb = theta_cmb;
  tf->growth_k0 = growth_k0;
  tf->alpha_gamma = sqrt(alpha_nu);
  tf->sound_horizon_fit = sound_horizon_fit;
  tf->beta_c = 1 / (1 - 0.949 * f_baryon);
  tf->growth_to_z0 = growth_to_z0;
}

static double eh_transfer(double kk, const eh_parms *tf) { /* :154-207, kk in 1/Mpc */
  const double qq = kk / tf->omhh * SQ(tf->theta_cmb);
  const double x = kk * tf->sound_horizon_fit * 0.43;
  const double gamma_eff = tf->omhh * (tf->alpha_gamma + (1 - tf->alpha_gamma) / (1 + SQ(SQ(x))));
  const double qq_eff = qq * tf->omhh / gamma_eff;
  const double tf_sup_L = log(2.71828 + 1.84 * tf->beta_c * tf->alpha_gamma * qq_eff);
  const double tf_sup_C = 14.4 + 325 / (1 + 60.5 * pow(qq_eff, 1.11));
  return tf_sup_L / (tf_sup_L + tf_sup_C * SQ(qq_eff));
}

typedef struct {
  const sf21o_hparams *p;
  eh_parms tf;
  double R;
} sig_ctx;

static double power_z0(double k, const sig_ctx *s) { /* powerFunction :316-330, k in h/Mpc */
  const double deltaH = 4.2E-5;
  const double tfk = eh_transfer(k * s->p->hubble, &s->tf);
  return s->tf.growth_to_z0 * s->tf.growth_to_z0 *
         (pow((1 / k), 3) * 2 * pow(H_PI * deltaH, 2) * pow((k * s->p->hubble), s->p->n_index + 3) * pow(tfk, 2));
}

static double j1_over_x(double x) { /* shared by W2 and W_filter, :335-359 */
  if (x < 0.03) return (1.0 / 3.0 - x * x * 1.0 / 30.0);
  return -(cos(x) - (sin(x) / x)) / x / x;
}
static double W2(double x) {
  const double j = j1_over_x(x);
  return 9.0 * j * j;
}
static double W_filter(double x) { return 3.0 * j1_over_x(x); }

static double dsigma(double x, void *vp) { /* dsigmaR :366-374 */
  const sig_ctx *s = (const sig_ctx *)vp;
  const double R = s->R;
  return (power_z0(x / R, s) / (2 * H_PI * H_PI) * (pow(x / R, 3)) * W2(x) / x +
          power_z0(1 / x / R, s) / (2 * H_PI * H_PI) * (pow(1 / x / R, 3)) * W2(1 / x) / x);
}

static double sigma_R(const sf21o_hparams *p, double R) { /* sigmaR :377-398 */
  sig_ctx s;
  s.p = p;
  s.R = R;
  eh_set(p, 0.0, &s.tf);
  gsl_integration_workspace *w = gsl_integration_workspace_alloc(1000);
  gsl_function F;
  F.function = &dsigma;
  F.params = &s;
  double res = 0, err = 0;
  gsl_integration_qag(&F, 0., 1., 0., 3e-7, 1000, GSL_INTEG_GAUSS15, w, &res, &err);
  gsl_integration_workspace_free(w);
  return sqrt(res);
}

double sf21o_h_sigma(const sf21o_hparams *p, double R) { /* sigma :415-424 */
  const double sig8_old = sigma_R(p, 8.0);
  return p->sig8 / sig8_old * sigma_R(p, R);
}

static double delta_filter(const sf21o_hparams *p, double sigma_aux, double growth) { /* :429-441 */
  const double dz = p->delta_c / growth;
  return sqrt(p->STa) * dz * (1.0 + p->STb * pow((sigma_aux * sigma_aux / (p->STa * dz * dz)), p->STc));
}

static double Hz(const sf21o_hparams *p, double z) { /* :224-226 */
  return p->hubble * H_H0 * sqrt(p->omega_m * (1. + z) * (1. + z) * (1. + z) + p->omega_l);
}

static double int_growth(const sf21o_hparams *p, double zz) { /* :242-257 */
  const double dz = 0.001;
  double intg = 0., z;
  const double hz0 = Hz(p, 0.);
  for (z = zz + dz / 2.; z < zz + 100.; z += dz) {
    const double hub = Hz(p, z) / hz0;
    intg += (1. + z) / hub / hub / hub;
  }
  return intg * dz;
}

double sf21o_h_growth(const sf21o_hparams *p, double z) { /* :262-266 */
  return Hz(p, z) / Hz(p, 0) * int_growth(p, z) / int_growth(p, 0.);
}

static double mass_to_radius(const sf21o_hparams *p, double M) { /* :498-500 */
  return pow(3 * M / (4 * H_PI * p->omega_m * H_RHO0 / p->hubble), 1.0 / 3.0);
}

double sf21o_h_mass_function(const sf21o_hparams *p, double z, double M) { /* :507-532 */
  const double M2 = M + (M / 1000.);
  const double a = 0.73, A = 0.353, pp = 0.175, E = 2.71828182846;
  const double R1 = mass_to_radius(p, M), R2 = mass_to_radius(p, M2);
  const double growth = sf21o_h_growth(p, z);
  const double deltac = p->delta_c;
  const double sigmaM = sf21o_h_sigma(p, R1) * growth;
  const double sigmaMdm = sf21o_h_sigma(p, R2) * growth;
  const double dlnsigmadm = (sigmaMdm - sigmaM) / (M / 1000.);
  const double nuhat = sqrt(a) * deltac / sigmaM;
  return (-p->omega_m * H_RHO0 / p->hubble) / M * dlnsigmadm / sigmaM * sqrt(2.0 / H_PI) * A *
         (1 + pow(nuhat, -2 * pp)) * nuhat * pow(E, -nuhat * nuhat / 2.0);
}

double sf21o_h_bias(const sf21o_hparams *p, double z, double sigmaM) { /* :446-458 */
  const double deltac = p->delta_c;
  const double growth = sf21o_h_growth(p, z);
  sigmaM = sigmaM * growth;
  const double nuhat = deltac / sigmaM;
  return (1.0 + ((nuhat * nuhat - 1.0) / deltac)) *
         pow((1.0 + (1 / (2.0 * pow(nuhat, 4)))), 0.06 - 0.02 * p->n_index);
}

/* ---- derived quantities (Input_variables.c:119-130) -------------------------- */
static double rho_m(const sf21o_hparams *p) { return p->omega_m * H_RHO0 / p->hubble; }
static double dx_halo(const sf21o_hparams *p) { return p->L / p->N; }

int sf21o_halo_schedule(const sf21o_hparams *p, double z, sf21o_hmass *out, int cap) {
  const double rhom = rho_m(p), dx = dx_halo(p), L3 = p->L * p->L * p->L;
  const double mass_dx = rhom * pow(dx, 3) * pow(10.0, p->dlm); /* :159 */
  const double growth = sf21o_h_growth(p, z);
  double R = p->L / 2.0; /* global_halo_Rmax */
  double M = (4.0 / 3.0) * H_PI * rhom * pow(R, 3);
  int n = 0;
  while (M > mass_dx && M >= p->Mmin) { /* :197 */
    const double dndm = sf21o_h_mass_function(p, z, M) * M * (pow(10.0, p->dlm) - 1) * L3;
    if (n < cap) {
      out[n].M = M;
      out[n].R = R;
      out[n].dndm = dndm;
      out[n].active = dndm > -log(1 - 0.1);
      out[n].dcmz = out[n].active ? growth * delta_filter(p, sf21o_h_sigma(p, R), growth) : 0.0;
    }
    n++;
    M = M / pow(10.0, p->dlm); /* :285-286 */
    R = pow(3 / 4.0 / H_PI / rhom * M, 1.0 / 3);
  }
  return n;
}

/* ---- filtered field of one mass (:211-229) ------------------------------------ */
typedef struct {
  long N, nh;
  fftwf_complex *spec; /* r2c of delta_z0, N x N x (N/2+1) */
  fftwf_complex *aux;  /* filtered spectrum, inverted in place (padded rows) */
  fftwf_plan c2r;
} hfield;

static int hfield_init(const sf21o_hparams *p, const float *delta_z0, hfield *h) {
  const long N = p->N, nh = N / 2 + 1;
  memset(h, 0, sizeof(*h));
  h->N = N;
  h->nh = nh;
  fftwf_plan_with_nthreads(p->nthreads > 0 ? p->nthreads : 1);
  float *in = fftwf_malloc(sizeof(float) * N * N * N);
  h->spec = fftwf_malloc(sizeof(fftwf_complex) * N * N * nh);
  h->aux = fftwf_malloc(sizeof(fftwf_complex) * N * N * nh);
  if (!in || !h->spec || !h->aux) return -1;
  memcpy(in, delta_z0, sizeof(float) * N * N * N);
  fftwf_plan r2c = fftwf_plan_dft_r2c_3d((int)N, (int)N, (int)N, in, h->spec, FFTW_ESTIMATE);
  h->c2r = fftwf_plan_dft_c2r_3d((int)N, (int)N, (int)N, h->aux, (float *)h->aux, FFTW_MEASURE);
  if (!r2c || !h->c2r) return -1;
  fftwf_execute(r2c);
  fftwf_destroy_plan(r2c);
  fftwf_free(in);
  return 0;
}

static void hfield_free(hfield *h) {
  if (h->c2r) fftwf_destroy_plan(h->c2r);
  fftwf_free(h->spec);
  fftwf_free(h->aux);
}

/* filter with radius R and the growth factor, inverse transform in place;
 * the field is then ((float *)aux)[(i N + j) 2 nh + p] */
static void hfield_run(const sf21o_hparams *p, hfield *h, double R, double growth) {
  const long N = h->N, nh = h->nh;
  const double dx = dx_halo(p), L3 = p->L * p->L * p->L, dk = 2 * H_PI / p->L;
#pragma omp parallel for num_threads(p->nthreads > 0 ? p->nthreads : 1)
  for (long i = 0; i < N; i++) {
    const long indi = i > N / 2 ? -(N - i) : i;
    for (long j = 0; j < N; j++) {
      const long indj = j > N / 2 ? -(N - j) : j;
      for (long q = 0; q <= N / 2; q++) {
        const double kk = dk * sqrt(indi * indi + indj * indj + q * q);
        const long t = i * N * nh + j * nh + q;
        h->aux[t] = h->spec[t] * W_filter(kk * R) * dx * dx * dx / L3 * growth;
      }
    }
  }
  fftwf_execute(h->c2r);
}

int sf21o_halo_field(const sf21o_hparams *p, double z, const float *delta_z0, int m, float *out) {
  sf21o_hmass *ms = malloc(sizeof(sf21o_hmass) * 256);
  const int nm = sf21o_halo_schedule(p, z, ms, 256);
  if (m < 0 || m >= nm || m >= 256) {
    free(ms);
    return -1;
  }
  hfield h;
  if (hfield_init(p, delta_z0, &h)) {
    hfield_free(&h);
    free(ms);
    return -1;
  }
  hfield_run(p, &h, ms[m].R, sf21o_h_growth(p, z));
  const long N = h.N;
  const float *f = (const float *)h.aux;
  for (long r = 0; r < N * N; r++) memcpy(out + r * N, f + r * 2 * h.nh, sizeof(float) * N);
  hfield_free(&h);
  free(ms);
  return 0;
}

void sf21o_taus_seed(unsigned long seed, unsigned long rng[3]) {
  gsl_rng *g = gsl_rng_alloc(gsl_rng_taus);
  gsl_rng_set(g, seed);
  rng[0] = g->s1;
  rng[1] = g->s2;
  rng[2] = g->s3;
  gsl_rng_free(g);
}

static long wrap(long x, long N) { /* check_borders :537-545 */
  x = x % N;
  if (x < 0) x += N;
  return x;
}

typedef struct {
  sf21o_halo *out;
  long cap, n;
} hcat;

static void emit(hcat *c, long i, long j, long q, double M) {
  if (c->n < c->cap) {
    c->out[c->n].x = i;
    c->out[c->n].y = j;
    c->out[c->n].z = q;
    c->out[c->n].Mass = M;
  }
  c->n++;
}

long sf21o_halo_find_z(const sf21o_hparams *p, double z, const float *delta_z0, sf21o_halo *out, long cap,
                       unsigned long rng[3], const uint32_t *const *masks, long *counts) {
  const long N = p->N, N3 = N * N * N;
  const double rhom = rho_m(p), dx = dx_halo(p);
  const double growth = sf21o_h_growth(p, z);
  sf21o_hmass ms[256];
  const int nm = sf21o_halo_schedule(p, z, ms, 256);
  if (nm > 256) return -1;
  char *flag = calloc((size_t)N3, 1);
  long *ind = malloc(sizeof(long) * (N3 / 200 > 1024 ? N3 / 200 : 1024));
  const long ind_cap = N3 / 200 > 1024 ? N3 / 200 : 1024;
  hfield h;
  memset(&h, 0, sizeof(h));
  if (!flag || !ind || (!masks && hfield_init(p, delta_z0, &h))) {
    hfield_free(&h);
    free(flag);
    free(ind);
    return -1;
  }
  hcat cat = {out, cap, 0};
  for (int m = 0; m < nm; m++) {
    long found = 0;
    if (ms[m].active) {
      const double R = ms[m].R, R2 = R * R, dcmz = ms[m].dcmz;
      const float *fld = NULL;
      if (!masks) {
        hfield_run(p, &h, R, growth);
        fld = (const float *)h.aux;
      }
      long nc = (long)(R / dx); /* :232-233 */
      if (nc == 0) nc = 1;
      for (long i = 0; i < N; i++)
        for (long j = 0; j < N; j++)
          for (long q = 0; q < N; q++) {
            const long t = (i * N + j) * N + q;
            const int cand = masks ? (int)((masks[m][t >> 5] >> (t & 31)) & 1u)
                                   : fld[i * 2 * h.nh * N + j * 2 * h.nh + q] > dcmz;
            if (!cand) continue;
            /* overlap test (:244-268), same loop order and early exit */
            int hit = 0;
            long k = 0;
            for (long ii = -nc; ii <= nc && !hit; ii++) {
              const double x2 = ii * ii * dx * dx;
              const long a = wrap(i + ii, N);
              for (long jj = -nc; jj <= nc && !hit; jj++) {
                const double y2 = jj * jj * dx * dx;
                if (x2 + y2 <= R2) {
                  const long b = wrap(j + jj, N);
                  for (long pp = -nc; pp <= nc && !hit; pp++) {
                    const double z2 = pp * dx * pp * dx;
                    if (x2 + y2 + z2 <= R2) {
                      const long c = wrap(q + pp, N);
                      const long u = a * N * N + b * N + c;
                      if (flag[u] != 1) {
                        if (k >= ind_cap) { /* the reference's list holds N^3/200 entries */
                          hfield_free(&h);
                          free(flag);
                          free(ind);
                          return -2;
                        }
                        ind[k++] = u;
                      } else
                        hit = 1;
                    }
                  }
                }
              }
            }
            if (!hit) {
              for (long u = 0; u < k; u++) flag[ind[u]] = 1;
              emit(&cat, i, j, q, ms[m].M);
              found++;
            }
          }
    }
    if (counts) counts[m] = found;
  }
  /* cell-size cycle (:293-321) */
  double M = rhom * pow(dx, 3);
  long ncell = 0;
  if (M >= p->Mmin) {
    const double R = pow(3 / 4.0 / H_PI / rhom * M, 1.0 / 3);
    const double dcmz = growth * delta_filter(p, sf21o_h_sigma(p, R), growth);
    for (long t = 0; t < N3; t++)
      if (flag[t] == 0 && delta_z0[t] * growth > dcmz) {
        flag[t] = 1;
        emit(&cat, t / (N * N), (t / N) % N, t % N, M);
        ncell++;
      }
  }
  if (counts) counts[nm] = ncell;
  M = M / pow(10.0, p->dlm);
  double R = pow(3 / 4.0 / H_PI / rhom * M, 1.0 / 3);
  /* subgrid cycle (:326-371) */
  if (p->use_sgrid == 1) {
    gsl_rng *g = gsl_rng_alloc(gsl_rng_taus);
    g->s1 = rng[0];
    g->s2 = rng[1];
    g->s3 = rng[2];
    while (M >= p->Mmin) {
      const double sigma_aux = sf21o_h_sigma(p, R);
      const double dndm = sf21o_h_mass_function(p, z, M) * M * (pow(10.0, p->dlm) - 1) * pow(dx, 3);
      const double hbias = sf21o_h_bias(p, z, sigma_aux);
      for (long t = 0; t < N3; t++) {
        if (flag[t] != 0) continue;
        const double tempv = delta_z0[t] * growth * hbias;
        const double Pn = gsl_ran_poisson(g, dndm);
        const int nn = (int)round(Pn * (1.0 + tempv));
        for (int u = 0; u < nn; u++) emit(&cat, t / (N * N), (t / N) % N, t % N, M);
      }
      M = M / pow(10.0, p->dlm);
      R = pow(3 / 4.0 / H_PI / rhom * M, 1.0 / 3);
    }
    rng[0] = g->s1;
    rng[1] = g->s2;
    rng[2] = g->s3;
    gsl_rng_free(g);
  }
  hfield_free(&h);
  free(flag);
  free(ind);
  return cat.n;
}
