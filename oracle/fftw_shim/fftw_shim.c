/*
 * Single-precision 3D real FFTs behind the FFTW3 API (see fftw3.h).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY: used to build the reference's own
 * get_HIIbubbles.c (oracle/_ref) and the CPU restatement oracle/hii_oracle.c.
 * It never ships in the GPU product library.
 *
 * Algorithm (the published mixed-radix Stockham autosort DFT):
 *   for each radix R of n (4,2,3,5, then any odd prime), with Ns = product
 *   of the radices already applied:
 *     v[r] = x[j + r n/R] * w^(r (j mod Ns) n/(Ns R)),  r = 0..R-1
 *     V = DFT_R(v)
 *     y[(j/Ns) Ns R + (j mod Ns) + r Ns] = V[r]
 * Arithmetic is float, twiddles are computed in double and rounded once.
 * r2c/c2r along the last axis use the half-length complex packing
 * (x[2m] + i x[2m+1]) for even n2.  The other axes are complex transforms
 * over gathered column blocks.  OpenMP threads split the independent lines
 * (the reference's FFTW is OpenMP-threaded as well, makefile:8,14).
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fftw3.h"

#define SHIM_PI 3.14159265358979323846

typedef struct {
  float re, im;
} cpx;

typedef struct {
  int n;
  int nf;
  int fac[40];
  cpx *tw;  /* tw[t] = exp(-2 pi i t / n), t in [0, n) */
  cpx *rtw; /* generic-radix tables: exp(-2 pi i q / R) for each prime R > 5 */
  int rtw_off[40];
} line_plan;

struct sf21_shim_plan_s {
  int kind; /* 0 = r2c, 1 = c2r */
  int n0, n1, n2, n2h;
  float *real;
  cpx *cplx;
  line_plan p0, p1, p2, p2half;
};

static int g_nthreads = 1;

void *fftwf_malloc(size_t n) {
  void *p = NULL;
  if (n == 0) n = 1;
  if (posix_memalign(&p, 64, n) != 0) return NULL;
  return p;
}
void fftwf_free(void *p) { free(p); }
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int nthreads) {
  g_nthreads = nthreads > 0 ? nthreads : 1;
}
void fftwf_cleanup_threads(void) {}

static int line_plan_init(line_plan *lp, int n) {
  int m = n, nf = 0;
  memset(lp, 0, sizeof(*lp));
  lp->n = n;
  if (n <= 0) return -1;
  while (m % 4 == 0) { lp->fac[nf++] = 4; m /= 4; }
  while (m % 2 == 0) { lp->fac[nf++] = 2; m /= 2; }
  while (m % 3 == 0) { lp->fac[nf++] = 3; m /= 3; }
  while (m % 5 == 0) { lp->fac[nf++] = 5; m /= 5; }
  for (int p = 7; m > 1; p += 2)
    while (m % p == 0) { lp->fac[nf++] = p; m /= p; }
  lp->nf = nf;
  for (int f = 0; f < nf; f++)
    if (lp->fac[f] > 64) return -1; /* prime factors above 64 unsupported */
  lp->tw = (cpx *)malloc(sizeof(cpx) * (size_t)n);
  if (!lp->tw) return -1;
  for (int t = 0; t < n; t++) {
    double a = -2.0 * SHIM_PI * (double)t / (double)n;
    lp->tw[t].re = (float)cos(a);
    lp->tw[t].im = (float)sin(a);
  }
  int tot = 0;
  for (int f = 0; f < nf; f++) {
    lp->rtw_off[f] = tot;
    if (lp->fac[f] > 5) tot += lp->fac[f];
  }
  if (tot > 0) {
    lp->rtw = (cpx *)malloc(sizeof(cpx) * (size_t)tot);
    if (!lp->rtw) return -1;
    for (int f = 0; f < nf; f++) {
      int R = lp->fac[f];
      if (R <= 5) continue;
      for (int q = 0; q < R; q++) {
        double a = -2.0 * SHIM_PI * (double)q / (double)R;
        lp->rtw[lp->rtw_off[f] + q].re = (float)cos(a);
        lp->rtw[lp->rtw_off[f] + q].im = (float)sin(a);
      }
    }
  }
  return 0;
}

static void line_plan_free(line_plan *lp) {
  free(lp->tw);
  free(lp->rtw);
}

/* twiddle exp(sign * 2 pi i t / n), sign = -1 forward, +1 inverse */
static inline cpx twf(const line_plan *lp, long t, int sign) {
  cpx w = lp->tw[t % lp->n];
  if (sign > 0) w.im = -w.im;
  return w;
}

static inline cpx cmul(cpx a, cpx b) {
  cpx r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

/* One complex line of length lp->n; x is overwritten, y is scratch of n. */
static void line_fft(const line_plan *lp, cpx *x, cpx *y, int sign) {
  const int n = lp->n;
  int Ns = 1;
  cpx *src = x, *dst = y;
  const float s = (float)sign;
  for (int f = 0; f < lp->nf; f++) {
    const int R = lp->fac[f];
    const int nR = n / R;
    const long tstep = n / (Ns * R);
    for (int j = 0; j < nR; j++) {
      const int jm = j % Ns;
      const int base = (j / Ns) * Ns * R + jm;
      cpx v[64];
      for (int r = 0; r < R; r++) {
        cpx a = src[j + r * nR];
        if (jm != 0 && r != 0) a = cmul(a, twf(lp, (long)jm * r * tstep, sign));
        v[r] = a;
      }
      if (R == 2) {
        cpx a = v[0], b = v[1];
        dst[base].re = a.re + b.re; dst[base].im = a.im + b.im;
        dst[base + Ns].re = a.re - b.re; dst[base + Ns].im = a.im - b.im;
      } else if (R == 4) {
        cpx t0, t1, t2, t3;
        t0.re = v[0].re + v[2].re; t0.im = v[0].im + v[2].im;
        t1.re = v[0].re - v[2].re; t1.im = v[0].im - v[2].im;
        t2.re = v[1].re + v[3].re; t2.im = v[1].im + v[3].im;
        t3.re = v[1].re - v[3].re; t3.im = v[1].im - v[3].im;
        /* multiply t3 by (sign) i : forward -i, inverse +i */
        cpx t3r;
        t3r.re = -s * t3.im;
        t3r.im = s * t3.re;
        dst[base].re = t0.re + t2.re; dst[base].im = t0.im + t2.im;
        dst[base + Ns].re = t1.re + t3r.re; dst[base + Ns].im = t1.im + t3r.im;
        dst[base + 2 * Ns].re = t0.re - t2.re; dst[base + 2 * Ns].im = t0.im - t2.im;
        dst[base + 3 * Ns].re = t1.re - t3r.re; dst[base + 3 * Ns].im = t1.im - t3r.im;
      } else if (R == 3) {
        const float c = -0.5f;
        const float sn = s * 0.86602540378443864676f; /* sign * sin(pi/3) */
        cpx a = v[0], b = v[1], d = v[2];
        float sr = b.re + d.re, si = b.im + d.im;
        float dr = b.re - d.re, di = b.im - d.im;
        dst[base].re = a.re + sr; dst[base].im = a.im + si;
        float mr = a.re + c * sr, mi = a.im + c * si;
        /* X1 = m + sign*i*sin60*(b-d), X2 = m - sign*i*sin60*(b-d) */
        dst[base + Ns].re = mr - sn * di; dst[base + Ns].im = mi + sn * dr;
        dst[base + 2 * Ns].re = mr + sn * di; dst[base + 2 * Ns].im = mi - sn * dr;
      } else {
        /* generic DFT of prime length R (5 and above) */
        const cpx *rt = NULL;
        cpx rloc[5];
        if (R == 5) {
          for (int q = 0; q < 5; q++) {
            double a = -2.0 * SHIM_PI * (double)q / 5.0;
            rloc[q].re = (float)cos(a);
            rloc[q].im = (float)sin(a);
          }
          rt = rloc;
        } else {
          rt = lp->rtw + lp->rtw_off[f];
        }
        for (int k = 0; k < R; k++) {
          cpx acc = v[0];
          for (int q = 1; q < R; q++) {
            cpx w = rt[(q * k) % R];
            if (sign > 0) w.im = -w.im;
            cpx p = cmul(v[q], w);
            acc.re += p.re;
            acc.im += p.im;
          }
          dst[base + k * Ns] = acc;
        }
      }
    }
    cpx *t = src; src = dst; dst = t;
    Ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(cpx) * (size_t)n);
}

static int plan_common(struct sf21_shim_plan_s *p, int n0, int n1, int n2) {
  if (n0 <= 0 || n1 <= 0 || n2 <= 0) return -1;
  p->n0 = n0; p->n1 = n1; p->n2 = n2; p->n2h = n2 / 2 + 1;
  if (line_plan_init(&p->p0, n0) || line_plan_init(&p->p1, n1) ||
      line_plan_init(&p->p2, n2))
    return -1;
  if (n2 % 2 == 0) {
    if (line_plan_init(&p->p2half, n2 / 2)) return -1;
  }
  return 0;
}

fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in,
                                 fftwf_complex *out, unsigned flags) {
  (void)flags;
  struct sf21_shim_plan_s *p = calloc(1, sizeof(*p));
  if (!p) return NULL;
  if (plan_common(p, n0, n1, n2)) { free(p); return NULL; }
  p->kind = 0;
  p->real = in;
  p->cplx = (cpx *)out;
  return p;
}

fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in,
                                 float *out, unsigned flags) {
  (void)flags;
  struct sf21_shim_plan_s *p = calloc(1, sizeof(*p));
  if (!p) return NULL;
  if (plan_common(p, n0, n1, n2)) { free(p); return NULL; }
  p->kind = 1;
  p->real = out;
  p->cplx = (cpx *)in;
  return p;
}

void fftwf_destroy_plan(fftwf_plan p) {
  if (!p) return;
  line_plan_free(&p->p0);
  line_plan_free(&p->p1);
  line_plan_free(&p->p2);
  line_plan_free(&p->p2half);
  free(p);
}

/* real row (length n) -> n/2+1 complex, forward, unnormalised */
static void row_r2c(const struct sf21_shim_plan_s *p, const float *x, cpx *X,
                    cpx *buf, cpx *scr) {
  const int n = p->n2;
  if (n % 2 == 0) {
    const int M = n / 2;
    for (int m = 0; m < M; m++) { buf[m].re = x[2 * m]; buf[m].im = x[2 * m + 1]; }
    line_fft(&p->p2half, buf, scr, -1);
    for (int k = 0; k <= M; k++) {
      cpx zk = buf[k % M];
      cpx zc = buf[(M - k) % M];
      zc.im = -zc.im; /* conj(Z[M-k]) */
      cpx E, O;
      E.re = 0.5f * (zk.re + zc.re); E.im = 0.5f * (zk.im + zc.im);
      /* O = (zk - zc) / (2i) = (d.im/2, -d.re/2) */
      float dr = zk.re - zc.re, di = zk.im - zc.im;
      O.re = 0.5f * di; O.im = -0.5f * dr;
      cpx w = p->p2.tw[k % n];
      cpx t = cmul(w, O);
      X[k].re = E.re + t.re; X[k].im = E.im + t.im;
    }
  } else {
    for (int m = 0; m < n; m++) { buf[m].re = x[m]; buf[m].im = 0.f; }
    line_fft(&p->p2, buf, scr, -1);
    for (int k = 0; k < p->n2h; k++) X[k] = buf[k];
  }
}

/* n/2+1 Hermitian complex -> real row, inverse, unnormalised */
static void row_c2r(const struct sf21_shim_plan_s *p, const cpx *X, float *x,
                    cpx *buf, cpx *scr) {
  const int n = p->n2;
  if (n % 2 == 0) {
    const int M = n / 2;
    for (int k = 0; k < M; k++) {
      cpx a = X[k];
      cpx b = X[M - k];
      b.im = -b.im; /* conj(X[M-k]) */
      cpx sum, dif;
      sum.re = a.re + b.re; sum.im = a.im + b.im;
      dif.re = a.re - b.re; dif.im = a.im - b.im;
      cpx w = p->p2.tw[k % n];
      w.im = -w.im; /* W^{-k} = exp(+2 pi i k / n) */
      cpx t = cmul(dif, w);
      /* Y = sum + i t */
      buf[k].re = sum.re - t.im;
      buf[k].im = sum.im + t.re;
    }
    line_fft(&p->p2half, buf, scr, +1);
    for (int m = 0; m < M; m++) { x[2 * m] = buf[m].re; x[2 * m + 1] = buf[m].im; }
  } else {
    /* rebuild the full Hermitian line */
    for (int k = 0; k < p->n2h; k++) buf[k] = X[k];
    for (int k = p->n2h; k < n; k++) { buf[k] = X[n - k]; buf[k].im = -buf[k].im; }
    line_fft(&p->p2, buf, scr, +1);
    for (int m = 0; m < n; m++) x[m] = buf[m].re;
  }
}

#define COLBLK 16

/* complex transform along a strided axis of a (n_outer, len, inner) array */
static void axis_fft(const line_plan *lp, cpx *data, long n_outer, int len,
                     long inner, int sign) {
  const long nblk = (inner + COLBLK - 1) / COLBLK;
  const long total = n_outer * nblk;
#pragma omp parallel num_threads(g_nthreads)
  {
    cpx *blk = (cpx *)malloc(sizeof(cpx) * (size_t)len * COLBLK);
    cpx *scr = (cpx *)malloc(sizeof(cpx) * (size_t)len);
#pragma omp for schedule(static)
    for (long t = 0; t < total; t++) {
      long o = t / nblk;
      long c0 = (t % nblk) * COLBLK;
      int w = (int)((inner - c0) < COLBLK ? (inner - c0) : COLBLK);
      cpx *base = data + o * (long)len * inner + c0;
      for (int l = 0; l < len; l++)
        for (int c = 0; c < w; c++) blk[c * len + l] = base[(long)l * inner + c];
      for (int c = 0; c < w; c++) line_fft(lp, blk + c * len, scr, sign);
      for (int l = 0; l < len; l++)
        for (int c = 0; c < w; c++) base[(long)l * inner + c] = blk[c * len + l];
    }
    free(blk);
    free(scr);
  }
}

void fftwf_execute(const fftwf_plan p) {
  const long n0 = p->n0, n1 = p->n1, n2h = p->n2h;
  const long rows = n0 * n1;
  if (p->kind == 0) {
#pragma omp parallel num_threads(g_nthreads)
    {
      cpx *buf = (cpx *)malloc(sizeof(cpx) * (size_t)p->n2);
      cpx *scr = (cpx *)malloc(sizeof(cpx) * (size_t)p->n2);
#pragma omp for schedule(static)
      for (long r = 0; r < rows; r++)
        row_r2c(p, p->real + r * p->n2, p->cplx + r * n2h, buf, scr);
      free(buf);
      free(scr);
    }
    axis_fft(&p->p1, p->cplx, n0, (int)n1, n2h, -1);
    axis_fft(&p->p0, p->cplx, 1, (int)n0, n1 * n2h, -1);
  } else {
    axis_fft(&p->p0, p->cplx, 1, (int)n0, n1 * n2h, +1);
    axis_fft(&p->p1, p->cplx, n0, (int)n1, n2h, +1);
#pragma omp parallel num_threads(g_nthreads)
    {
      cpx *buf = (cpx *)malloc(sizeof(cpx) * (size_t)p->n2);
      cpx *scr = (cpx *)malloc(sizeof(cpx) * (size_t)p->n2);
#pragma omp for schedule(static)
      for (long r = 0; r < rows; r++)
        row_c2r(p, p->cplx + r * n2h, p->real + r * p->n2, buf, scr);
      free(buf);
      free(scr);
    }
  }
}
