/*
 * Body of the FFTW-API shim, instantiated twice by fftw_shim.c (ORACLE /
 * TEST INFRASTRUCTURE ONLY): SREAL = float with the fftwf_ names and
 * SREAL = double with the fftw_ names.  See fftw_shim.c for the algorithm.
 */
typedef struct {
  SREAL re, im;
} SCPX;

typedef struct {
  int n;
  int nf;
  int fac[40];
  SCPX *tw;  /* tw[t] = exp(-2 pi i t / n), t in [0, n) */
  SCPX *rtw; /* generic-radix tables: exp(-2 pi i q / R) for each prime R > 5 */
  int rtw_off[40];
} S(line_plan);

struct SPLAN {
  int kind; /* 0 = r2c, 1 = c2r */
  int n0, n1, n2, n2h;
  long rs; /* real row stride: n2, or 2 (n2/2+1) for an in-place plan */
  SREAL *real;
  SCPX *cplx;
  S(line_plan) p0, p1, p2, p2half;
};

void *API(malloc)(size_t n) {
  void *p = NULL;
  if (n == 0) n = 1;
  if (posix_memalign(&p, 64, n) != 0) return NULL;
  return p;
}
void API(free)(void *p) { free(p); }
int API(init_threads)(void) { return 1; }
void API(plan_with_nthreads)(int nthreads) {
  g_nthreads = nthreads > 0 ? nthreads : 1;
}
void API(cleanup_threads)(void) {}

static int S(line_plan_init)(S(line_plan) *lp, int n) {
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
  lp->tw = (SCPX *)malloc(sizeof(SCPX) * (size_t)n);
  if (!lp->tw) return -1;
  for (int t = 0; t < n; t++) {
    double a = -2.0 * SHIM_PI * (double)t / (double)n;
    lp->tw[t].re = (SREAL)cos(a);
    lp->tw[t].im = (SREAL)sin(a);
  }
  int tot = 0;
  for (int f = 0; f < nf; f++) {
    lp->rtw_off[f] = tot;
    if (lp->fac[f] > 5) tot += lp->fac[f];
  }
  if (tot > 0) {
    lp->rtw = (SCPX *)malloc(sizeof(SCPX) * (size_t)tot);
    if (!lp->rtw) return -1;
    for (int f = 0; f < nf; f++) {
      int R = lp->fac[f];
      if (R <= 5) continue;
      for (int q = 0; q < R; q++) {
        double a = -2.0 * SHIM_PI * (double)q / (double)R;
        lp->rtw[lp->rtw_off[f] + q].re = (SREAL)cos(a);
        lp->rtw[lp->rtw_off[f] + q].im = (SREAL)sin(a);
      }
    }
  }
  return 0;
}

static void S(line_plan_free)(S(line_plan) *lp) {
  free(lp->tw);
  free(lp->rtw);
}

/* twiddle exp(sign * 2 pi i t / n), sign = -1 forward, +1 inverse */
static inline SCPX S(twf)(const S(line_plan) *lp, long t, int sign) {
  SCPX w = lp->tw[t % lp->n];
  if (sign > 0) w.im = -w.im;
  return w;
}

static inline SCPX S(cmul)(SCPX a, SCPX b) {
  SCPX r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

/* One complex line of length lp->n; x is overwritten, y is scratch of n. */
static void S(line_fft)(const S(line_plan) *lp, SCPX *x, SCPX *y, int sign) {
  const int n = lp->n;
  int Ns = 1;
  SCPX *src = x, *dst = y;
  const SREAL s = (SREAL)sign;
  for (int f = 0; f < lp->nf; f++) {
    const int R = lp->fac[f];
    const int nR = n / R;
    const long tstep = n / (Ns * R);
    for (int j = 0; j < nR; j++) {
      const int jm = j % Ns;
      const int base = (j / Ns) * Ns * R + jm;
      SCPX v[64];
      for (int r = 0; r < R; r++) {
        SCPX a = src[j + r * nR];
        if (jm != 0 && r != 0) a = S(cmul)(a, S(twf)(lp, (long)jm * r * tstep, sign));
        v[r] = a;
      }
      if (R == 2) {
        SCPX a = v[0], b = v[1];
        dst[base].re = a.re + b.re; dst[base].im = a.im + b.im;
        dst[base + Ns].re = a.re - b.re; dst[base + Ns].im = a.im - b.im;
      } else if (R == 4) {
        SCPX t0, t1, t2, t3;
        t0.re = v[0].re + v[2].re; t0.im = v[0].im + v[2].im;
        t1.re = v[0].re - v[2].re; t1.im = v[0].im - v[2].im;
        t2.re = v[1].re + v[3].re; t2.im = v[1].im + v[3].im;
        t3.re = v[1].re - v[3].re; t3.im = v[1].im - v[3].im;
        /* multiply t3 by (sign) i : forward -i, inverse +i */
        SCPX t3r;
        t3r.re = -s * t3.im;
        t3r.im = s * t3.re;
        dst[base].re = t0.re + t2.re; dst[base].im = t0.im + t2.im;
        dst[base + Ns].re = t1.re + t3r.re; dst[base + Ns].im = t1.im + t3r.im;
        dst[base + 2 * Ns].re = t0.re - t2.re; dst[base + 2 * Ns].im = t0.im - t2.im;
        dst[base + 3 * Ns].re = t1.re - t3r.re; dst[base + 3 * Ns].im = t1.im - t3r.im;
      } else if (R == 3) {
        const SREAL c = -((SREAL)0.5);
        const SREAL sn = s * ((SREAL)0.86602540378443864676); /* sign * sin(pi/3) */
        SCPX a = v[0], b = v[1], d = v[2];
        SREAL sr = b.re + d.re, si = b.im + d.im;
        SREAL dr = b.re - d.re, di = b.im - d.im;
        dst[base].re = a.re + sr; dst[base].im = a.im + si;
        SREAL mr = a.re + c * sr, mi = a.im + c * si;
        /* X1 = m + sign*i*sin60*(b-d), X2 = m - sign*i*sin60*(b-d) */
        dst[base + Ns].re = mr - sn * di; dst[base + Ns].im = mi + sn * dr;
        dst[base + 2 * Ns].re = mr + sn * di; dst[base + 2 * Ns].im = mi - sn * dr;
      } else {
        /* generic DFT of prime length R (5 and above) */
        const SCPX *rt = NULL;
        SCPX rloc[5];
        if (R == 5) {
          for (int q = 0; q < 5; q++) {
            double a = -2.0 * SHIM_PI * (double)q / 5.0;
            rloc[q].re = (SREAL)cos(a);
            rloc[q].im = (SREAL)sin(a);
          }
          rt = rloc;
        } else {
          rt = lp->rtw + lp->rtw_off[f];
        }
        for (int k = 0; k < R; k++) {
          SCPX acc = v[0];
          for (int q = 1; q < R; q++) {
            SCPX w = rt[(q * k) % R];
            if (sign > 0) w.im = -w.im;
            SCPX p = S(cmul)(v[q], w);
            acc.re += p.re;
            acc.im += p.im;
          }
          dst[base + k * Ns] = acc;
        }
      }
    }
    SCPX *t = src; src = dst; dst = t;
    Ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(SCPX) * (size_t)n);
}

static int S(plan_common)(struct SPLAN *p, int n0, int n1, int n2) {
  if (n0 <= 0 || n1 <= 0 || n2 <= 0) return -1;
  p->n0 = n0; p->n1 = n1; p->n2 = n2; p->n2h = n2 / 2 + 1;
  if (S(line_plan_init)(&p->p0, n0) || S(line_plan_init)(&p->p1, n1) ||
      S(line_plan_init)(&p->p2, n2))
    return -1;
  if (n2 % 2 == 0) {
    if (S(line_plan_init)(&p->p2half, n2 / 2)) return -1;
  }
  return 0;
}

SPLAN_T API(plan_dft_r2c_3d)(int n0, int n1, int n2, SREAL *in,
                                 SCOMPLEX_T *out, unsigned flags) {
  (void)flags;
  struct SPLAN *p = calloc(1, sizeof(*p));
  if (!p) return NULL;
  if (S(plan_common)(p, n0, n1, n2)) { free(p); return NULL; }
  p->kind = 0;
  p->real = in;
  p->cplx = (SCPX *)out;
  p->rs = ((void *)in == (void *)out) ? 2L * p->n2h : p->n2;
  return p;
}

SPLAN_T API(plan_dft_c2r_3d)(int n0, int n1, int n2, SCOMPLEX_T *in,
                                 SREAL *out, unsigned flags) {
  (void)flags;
  struct SPLAN *p = calloc(1, sizeof(*p));
  if (!p) return NULL;
  if (S(plan_common)(p, n0, n1, n2)) { free(p); return NULL; }
  p->kind = 1;
  p->real = out;
  p->cplx = (SCPX *)in;
  p->rs = ((void *)in == (void *)out) ? 2L * p->n2h : p->n2;
  return p;
}

void API(destroy_plan)(SPLAN_T p) {
  if (!p) return;
  S(line_plan_free)(&p->p0);
  S(line_plan_free)(&p->p1);
  S(line_plan_free)(&p->p2);
  S(line_plan_free)(&p->p2half);
  free(p);
}

/* real row (length n) -> n/2+1 complex, forward, unnormalised */
static void S(row_r2c)(const struct SPLAN *p, const SREAL *x, SCPX *X,
                    SCPX *buf, SCPX *scr) {
  const int n = p->n2;
  if (n % 2 == 0) {
    const int M = n / 2;
    for (int m = 0; m < M; m++) { buf[m].re = x[2 * m]; buf[m].im = x[2 * m + 1]; }
    S(line_fft)(&p->p2half, buf, scr, -1);
    for (int k = 0; k <= M; k++) {
      SCPX zk = buf[k % M];
      SCPX zc = buf[(M - k) % M];
      zc.im = -zc.im; /* conj(Z[M-k]) */
      SCPX E, O;
      E.re = ((SREAL)0.5) * (zk.re + zc.re); E.im = ((SREAL)0.5) * (zk.im + zc.im);
      /* O = (zk - zc) / (2i) = (d.im/2, -d.re/2) */
      SREAL dr = zk.re - zc.re, di = zk.im - zc.im;
      O.re = ((SREAL)0.5) * di; O.im = -((SREAL)0.5) * dr;
      SCPX w = p->p2.tw[k % n];
      SCPX t = S(cmul)(w, O);
      X[k].re = E.re + t.re; X[k].im = E.im + t.im;
    }
  } else {
    for (int m = 0; m < n; m++) { buf[m].re = x[m]; buf[m].im = ((SREAL)0.); }
    S(line_fft)(&p->p2, buf, scr, -1);
    for (int k = 0; k < p->n2h; k++) X[k] = buf[k];
  }
}

/* n/2+1 Hermitian complex -> real row, inverse, unnormalised */
static void S(row_c2r)(const struct SPLAN *p, const SCPX *X, SREAL *x,
                    SCPX *buf, SCPX *scr) {
  const int n = p->n2;
  if (n % 2 == 0) {
    const int M = n / 2;
    for (int k = 0; k < M; k++) {
      SCPX a = X[k];
      SCPX b = X[M - k];
      b.im = -b.im; /* conj(X[M-k]) */
      SCPX sum, dif;
      sum.re = a.re + b.re; sum.im = a.im + b.im;
      dif.re = a.re - b.re; dif.im = a.im - b.im;
      SCPX w = p->p2.tw[k % n];
      w.im = -w.im; /* W^{-k} = exp(+2 pi i k / n) */
      SCPX t = S(cmul)(dif, w);
      /* Y = sum + i t */
      buf[k].re = sum.re - t.im;
      buf[k].im = sum.im + t.re;
    }
    S(line_fft)(&p->p2half, buf, scr, +1);
    for (int m = 0; m < M; m++) { x[2 * m] = buf[m].re; x[2 * m + 1] = buf[m].im; }
  } else {
    /* rebuild the full Hermitian line */
    for (int k = 0; k < p->n2h; k++) buf[k] = X[k];
    for (int k = p->n2h; k < n; k++) { buf[k] = X[n - k]; buf[k].im = -buf[k].im; }
    S(line_fft)(&p->p2, buf, scr, +1);
    for (int m = 0; m < n; m++) x[m] = buf[m].re;
  }
}

/* complex transform along a strided axis of a (n_outer, len, inner) array */
static void S(axis_fft)(const S(line_plan) *lp, SCPX *data, long n_outer, int len,
                     long inner, int sign) {
  const long nblk = (inner + COLBLK - 1) / COLBLK;
  const long total = n_outer * nblk;
#pragma omp parallel num_threads(g_nthreads)
  {
    SCPX *blk = (SCPX *)malloc(sizeof(SCPX) * (size_t)len * COLBLK);
    SCPX *scr = (SCPX *)malloc(sizeof(SCPX) * (size_t)len);
#pragma omp for schedule(static)
    for (long t = 0; t < total; t++) {
      long o = t / nblk;
      long c0 = (t % nblk) * COLBLK;
      int w = (int)((inner - c0) < COLBLK ? (inner - c0) : COLBLK);
      SCPX *base = data + o * (long)len * inner + c0;
      for (int l = 0; l < len; l++)
        for (int c = 0; c < w; c++) blk[c * len + l] = base[(long)l * inner + c];
      for (int c = 0; c < w; c++) S(line_fft)(lp, blk + c * len, scr, sign);
      for (int l = 0; l < len; l++)
        for (int c = 0; c < w; c++) base[(long)l * inner + c] = blk[c * len + l];
    }
    free(blk);
    free(scr);
  }
}

void API(execute)(const SPLAN_T p) {
  const long n0 = p->n0, n1 = p->n1, n2h = p->n2h;
  const long rows = n0 * n1;
  if (p->kind == 0) {
#pragma omp parallel num_threads(g_nthreads)
    {
      SCPX *buf = (SCPX *)malloc(sizeof(SCPX) * (size_t)p->n2);
      SCPX *scr = (SCPX *)malloc(sizeof(SCPX) * (size_t)p->n2);
#pragma omp for schedule(static)
      for (long r = 0; r < rows; r++)
        S(row_r2c)(p, p->real + r * p->rs, p->cplx + r * n2h, buf, scr);
      free(buf);
      free(scr);
    }
    S(axis_fft)(&p->p1, p->cplx, n0, (int)n1, n2h, -1);
    S(axis_fft)(&p->p0, p->cplx, 1, (int)n0, n1 * n2h, -1);
  } else {
    S(axis_fft)(&p->p0, p->cplx, 1, (int)n0, n1 * n2h, +1);
    S(axis_fft)(&p->p1, p->cplx, n0, (int)n1, n2h, +1);
#pragma omp parallel num_threads(g_nthreads)
    {
      SCPX *buf = (SCPX *)malloc(sizeof(SCPX) * (size_t)p->n2);
      SCPX *scr = (SCPX *)malloc(sizeof(SCPX) * (size_t)p->n2);
#pragma omp for schedule(static)
      for (long r = 0; r < rows; r++)
        S(row_c2r)(p, p->cplx + r * n2h, p->real + r * p->rs, buf, scr);
      free(buf);
      free(scr);
    }
  }
}
