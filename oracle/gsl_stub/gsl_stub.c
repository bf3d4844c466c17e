/*
 * Restatements of the three GSL routines the reference reaches on the paths
 * this repository checks.  ORACLE / TEST INFRASTRUCTURE ONLY: GSL is not
 * installed here (the reference's makefile links -lgsl, version unpinned),
 * so the reference sources are built against these bodies.
 *
 *  - gsl_integration_qag with the 15-point Gauss-Kronrod rule
 *    (auxiliary.c:394-396, sigmaR): the published QUADPACK algorithm QAG
 *    (R. Piessens, E. de Doncker-Kapenga, C. Ueberhuber, D. Kahaner,
 *    "QUADPACK", Springer 1983): integrate the whole range with QK15; while
 *    the summed error estimate exceeds max(epsabs, epsrel |area|), bisect the
 *    subinterval with the largest error estimate, with QUADPACK's error
 *    rescaling, its two round-off counters and its too-small-interval stop;
 *    the result is the sum of the subinterval results in list order.
 *  - gsl_rng_taus / gsl_rng_uniform (get_halos.c:70-71): L'Ecuyer's
 *    three-component Tausworthe generator "taus88" (Math. Comp. 65 (1996)
 *    203-213) with GSL's documented seeding (seed 0 -> 1; each component
 *    seeded from the 69069 congruential sequence and raised to its minimum
 *    valid value; six warm-up draws); uniform = draw / 2^32.
 *  - gsl_ran_poisson (get_halos.c:353) for means <= 10: Knuth's product of
 *    uniforms (TAOCP vol. 2, 3.4.1): multiply uniforms until the product is
 *    at most exp(-mu); the count of factors minus one.
 * The rule's nodes and weights (Kronrod's 15-point extension of the 7-point
 * Gauss rule) are checked numerically by the CPU tests (exact integration of
 * polynomials up to degree 22, Gauss part against numpy's leggauss(7)).
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gsl/gsl_integration.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"

/* ---- QK15 ----------------------------------------------------------------- */
static const double qk15_x[8] = {  /* Kronrod abscissae; odd entries are the Gauss ones */
    0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
    0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
    0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
    0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
static const double qk15_wg[4] = {  /* 7-point Gauss weights (last = centre) */
    0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
    0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
static const double qk15_wk[8] = {  /* 15-point Kronrod weights (last = centre) */
    0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
    0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
    0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
    0.204432940075298892414161999234649, 0.209482141084727828012999174891714};

/* exported for the node/weight check */
const double *sf21o_qk15_nodes(int which) {
  return which == 0 ? qk15_x : which == 1 ? qk15_wg : qk15_wk;
}

static double qk_err_scale(double err, double res_abs, double res_asc) {
  err = fabs(err);
  if (res_asc != 0.0 && err != 0.0) {
    const double s = pow(200.0 * err / res_asc, 1.5);
    err = s < 1.0 ? res_asc * s : res_asc;
  }
  if (res_abs > DBL_MIN / (50.0 * DBL_EPSILON)) {
    const double floor_err = 50.0 * DBL_EPSILON * res_abs;
    if (floor_err > err) err = floor_err;
  }
  return err;
}

static void qk15(const gsl_function *f, double a, double b, double *res, double *err,
                 double *res_abs, double *res_asc) {
  double fv1[7], fv2[7];
  const double c = 0.5 * (a + b), h = 0.5 * (b - a), ah = fabs(h);
  const double fc = f->function(c, f->params);
  double rg = fc * qk15_wg[3];
  double rk = fc * qk15_wk[7];
  double ra = fabs(rk);
  for (int j = 0; j < 3; j++) { /* Gauss nodes */
    const int jj = 2 * j + 1;
    const double dx = h * qk15_x[jj];
    const double f1 = f->function(c - dx, f->params), f2 = f->function(c + dx, f->params);
    const double s = f1 + f2;
    fv1[jj] = f1;
    fv2[jj] = f2;
    rg += qk15_wg[j] * s;
    rk += qk15_wk[jj] * s;
    ra += qk15_wk[jj] * (fabs(f1) + fabs(f2));
  }
  for (int j = 0; j < 4; j++) { /* Kronrod-only nodes */
    const int jj = 2 * j;
    const double dx = h * qk15_x[jj];
    const double f1 = f->function(c - dx, f->params), f2 = f->function(c + dx, f->params);
    const double s = f1 + f2;
    fv1[jj] = f1;
    fv2[jj] = f2;
    rk += qk15_wk[jj] * s;
    ra += qk15_wk[jj] * (fabs(f1) + fabs(f2));
  }
  const double mean = rk * 0.5;
  double rasc = qk15_wk[7] * fabs(fc - mean);
  for (int j = 0; j < 7; j++) rasc += qk15_wk[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
  const double e = (rk - rg) * h;
  rk *= h;
  ra *= ah;
  rasc *= ah;
  *res = rk;
  *res_abs = ra;
  *res_asc = rasc;
  *err = qk_err_scale(e, ra, rasc);
}

/* ---- QAG ------------------------------------------------------------------ */
struct gsl_integration_workspace_s {
  size_t cap, n;
  double *lo, *hi, *r, *e;
};

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
  gsl_integration_workspace *w = calloc(1, sizeof(*w));
  if (!w || n == 0) {
    free(w);
    return NULL;
  }
  w->cap = n;
  w->lo = malloc(sizeof(double) * n);
  w->hi = malloc(sizeof(double) * n);
  w->r = malloc(sizeof(double) * n);
  w->e = malloc(sizeof(double) * n);
  if (!w->lo || !w->hi || !w->r || !w->e) {
    gsl_integration_workspace_free(w);
    return NULL;
  }
  return w;
}

void gsl_integration_workspace_free(gsl_integration_workspace *w) {
  if (!w) return;
  free(w->lo);
  free(w->hi);
  free(w->r);
  free(w->e);
  free(w);
}

static size_t qag_worst(const gsl_integration_workspace *w) {
  size_t m = 0;
  for (size_t k = 1; k < w->n; k++)
    if (w->e[k] > w->e[m]) m = k;
  return m;
}

int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                        size_t limit, int key, gsl_integration_workspace *w, double *result,
                        double *abserr) {
  if (key != GSL_INTEG_GAUSS15) {
    fprintf(stderr, "GSL stub: only the 15-point rule is restated\n");
    abort();
  }
  if (limit > w->cap) limit = w->cap;
  double r0, e0, ra0, rasc0;
  qk15(f, a, b, &r0, &e0, &ra0, &rasc0);
  w->n = 1;
  w->lo[0] = a;
  w->hi[0] = b;
  w->r[0] = r0;
  w->e[0] = e0;
  double tol = fmax(epsabs, epsrel * fabs(r0));
  const double round_off = 50.0 * DBL_EPSILON * ra0;
  *result = r0;
  *abserr = e0;
  if (e0 <= round_off && e0 > tol) return 18; /* round-off on the first attempt */
  if ((e0 <= tol && e0 != rasc0) || e0 == 0.0) return 0;
  if (limit == 1) return 11;
  double area = r0, errsum = e0;
  int ro1 = 0, ro2 = 0, stop = 0;
  size_t it = 1;
  do {
    const size_t m = qag_worst(w);
    const double lo = w->lo[m], hi = w->hi[m], rm = w->r[m], em = w->e[m];
    const double mid = 0.5 * (lo + hi);
    double r1, e1, ra1, rasc1, r2, e2, ra2, rasc2;
    qk15(f, lo, mid, &r1, &e1, &ra1, &rasc1);
    qk15(f, mid, hi, &r2, &e2, &ra2, &rasc2);
    const double r12 = r1 + r2, e12 = e1 + e2;
    errsum += e12 - em;
    area += r12 - rm;
    if (rasc1 != e1 && rasc2 != e2) {
      if (fabs(rm - r12) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * em) ro1++;
      if (it >= 10 && e12 > em) ro2++;
    }
    tol = fmax(epsabs, epsrel * fabs(area));
    if (errsum > tol) {
      if (ro1 >= 6 || ro2 >= 20) stop = 2;
      const double tiny = (1.0 + 100.0 * DBL_EPSILON) * (fabs(mid) + 1000.0 * DBL_MIN);
      if (fabs(lo) <= tiny && fabs(hi) <= tiny) stop = 3;
    }
    /* the half with the larger error keeps slot m, the other is appended */
    const size_t k = w->n++;
    if (e2 > e1) {
      w->lo[m] = mid; w->r[m] = r2; w->e[m] = e2;
      w->lo[k] = lo; w->hi[k] = mid; w->r[k] = r1; w->e[k] = e1;
    } else {
      w->hi[m] = mid; w->r[m] = r1; w->e[m] = e1;
      w->lo[k] = mid; w->hi[k] = hi; w->r[k] = r2; w->e[k] = e2;
    }
    it++;
  } while (it < limit && !stop && errsum > tol);
  double sum = 0.0;
  for (size_t k = 0; k < w->n; k++) sum += w->r[k];
  *result = sum;
  *abserr = errsum;
  if (errsum <= tol) return 0;
  return stop ? 18 : 11;
}

/* ---- taus88 ----------------------------------------------------------------- */
static const gsl_rng_type taus_type = {"taus"};
const gsl_rng_type *gsl_rng_taus = &taus_type;

#define SF21_M32 0xffffffffUL
static unsigned long taus_step(gsl_rng *g) {
  g->s1 = (((g->s1 & 4294967294UL) << 12) & SF21_M32) ^ ((((g->s1 << 13) & SF21_M32) ^ g->s1) >> 19);
  g->s2 = (((g->s2 & 4294967288UL) << 4) & SF21_M32) ^ ((((g->s2 << 2) & SF21_M32) ^ g->s2) >> 25);
  g->s3 = (((g->s3 & 4294967280UL) << 17) & SF21_M32) ^ ((((g->s3 << 3) & SF21_M32) ^ g->s3) >> 11);
  return g->s1 ^ g->s2 ^ g->s3;
}

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  gsl_rng *g = calloc(1, sizeof(*g));
  if (!g) return NULL;
  g->type = T;
  gsl_rng_set(g, 0);
  return g;
}

void gsl_rng_set(const gsl_rng *r, unsigned long int seed) {
  gsl_rng *g = (gsl_rng *)r;
  if (seed == 0) seed = 1;
  g->s1 = (69069UL * seed) & SF21_M32;
  if (g->s1 < 2) g->s1 += 2;
  g->s2 = (69069UL * g->s1) & SF21_M32;
  if (g->s2 < 8) g->s2 += 8;
  g->s3 = (69069UL * g->s2) & SF21_M32;
  if (g->s3 < 16) g->s3 += 16;
  for (int k = 0; k < 6; k++) taus_step(g);
}

void gsl_rng_free(gsl_rng *r) { free(r); }

unsigned long gsl_rng_get(const gsl_rng *r) { return taus_step((gsl_rng *)r); }

double gsl_rng_uniform(const gsl_rng *r) { return taus_step((gsl_rng *)r) / 4294967296.0; }

unsigned int gsl_ran_poisson(const gsl_rng *r, double mu) {
  if (mu > 10) {
    fprintf(stderr, "GSL stub: Poisson mean %g > 10 (the gamma/binomial branch is not restated)\n", mu);
    abort();
  }
  const double emu = exp(-mu);
  double prod = 1.0;
  unsigned int k = 0;
  do {
    prod *= gsl_rng_uniform(r);
    k++;
  } while (prod > emu);
  return k - 1;
}
