// Host-side check of prologue_fast.h: every fast path returns the same float
// as its exact soft-double chain whenever it returns at all.
// Usage: prologue_fast_check <n_random> <seed>
// Prints "<name> <cases> <mismatches> <fallbacks>" for
//   rrec_exhaustive: Rrec of every float in [0.5, 2) at z = 7 (L = 300 Mpc/h, N = 512);
//   rrec_lognormal:  Rrec of 1 + d for lognormal 1 + d (sigma 1.5), six redshifts, four boxes;
//   rrec_wide:       Rrec of floats with binary exponents in [-60, 60], same sweeps;
//   resid:           (1 + d) 1.881e-7 (1+z)^3 G_H(z) for the same densities and redshifts;
//   src:             the source products of both source kinds, positive floats of all sizes and zeros;
//   xhi_realistic:   XHI of the residual-fraction arguments above;
//   xhi_wide:        XHI of floats with binary exponents in [-40, 20].
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#include "prologue_fast.h"

static uint64_t d2bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
static uint32_t f2bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static float bits2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

static uint64_t rng_state;
static uint64_t rnd64() {
  rng_state ^= rng_state << 13; rng_state ^= rng_state >> 7; rng_state ^= rng_state << 17;
  return rng_state;
}
static double rnd_unit() { return (double)(rnd64() >> 11) * 0x1p-53; }
static float rnd_float_exp(int emin, int emax) {  // positive float, binary exponent in [emin, emax]
  const uint32_t e = (uint32_t)(127 + emin) + (uint32_t)(rnd64() % (uint64_t)(emax - emin + 1));
  return bits2f((e << 23) | ((uint32_t)rnd64() & 0x7FFFFFu));
}

// G_H(z) of the reference (user_functions.c), used only to make realistic constants
static double g_h(double z) {
  const double lo = -4.37152818e-05 * std::pow(z, 5.) + 1.64394635e-03 * std::pow(z, 4.) - 2.03044756e-02 * std::pow(z, 3.);
  const double hi = 7.18335221e-02 * std::pow(z, 2.) - 8.85791388e-02 * z - 1.20887500e+01;
  return 4.19232273531e-13 / std::pow(10.0, lo + hi);
}

struct Consts {  // the prologue's constants at redshift z for a box of side L (Mpc/h) and N cells
  sd_t rec1, dvv, r2, r3, v_norm, resid[3];
  sd_divc r2c, v_normc;
  RrecFast rf;
  ProdFast pf_resid;
  Consts(double z, double L, int N) {
    rec1 = d2bits(1.e-24 * 9.84815696 * std::pow(1.0 + z, 5.06773134));
    dvv = d2bits(std::pow(L * 3.0856775807e24 / N / 0.7 / (1. + z), 3.0));
    r2 = d2bits(1.76105133);
    r3 = d2bits(0.81722878);
    v_norm = d2bits(1.e+45);
    r2c = sd_divc_prepare(r2);
    v_normc = sd_divc_prepare(v_norm);
    rf = rrec_fast_prepare(rec1, dvv, v_norm, r2, r3);
    resid[0] = d2bits(1.881e-7);
    resid[1] = d2bits(std::pow(1. + z, 3.0));
    resid[2] = d2bits(g_h(z));
    pf_resid = prod_fast_prepare(resid, 3);
  }
};

struct Stat { const char* name; long n = 0, bad = 0, fallback = 0; };
static void tally(Stat& s, bool fast, float got, float want, double arg) {
  s.n++;
  if (!fast) {
    s.fallback++;
    return;
  }
  if (f2bits(got) != f2bits(want)) {
    if (s.bad < 5) printf("# %s mismatch arg=%a fast=%a exact=%a\n", s.name, arg, got, want);
    s.bad++;
  }
}

static void check_rrec(Stat& s, const Consts& c, float od) {
  float got = 0.f;
  const bool fast = rrec_fast(od, c.rf, &got);
  const float want = fast ? sd_to_float(rrec_exact(od, c.r2c, c.r3, c.rec1, c.dvv, c.v_normc)) : 0.f;
  tally(s, fast, got, want, od);
}

static void check_prod(Stat& s, sd_t x, const ProdFast& k, const sd_t* ks, int n) {
  float got = 0.f;
  const bool fast = prod_fast(x, k, &got);
  sd_t t = x;
  for (int i = 0; i < n; ++i) t = sd_mul(t, ks[i]);
  double xd;
  std::memcpy(&xd, &x, 8);
  tally(s, fast, got, sd_to_float(t), xd);
}

static void check_xhi(Stat& s, float ratio) {
  // the fast division's own decision, for the fallback count
  const sd_t r = sd_from_float(ratio);
  const sd_t two_r = sd_ldexp(r, 1);
  const sd_t b = sd_add(two_r, 0x3FF0000000000000ULL);
  const sd_t g = sd_sqrt_fast(sd_sub(sd_mul(b, b), sd_mul(sd_ldexp(r, 2), r)));
  float q;
  const bool fast = div_fast(sd_sub(b, g), two_r, &q);
  const float want = sd_to_float(xhi_exact(r));
  const float got = xhi_float(ratio);  // the device's function: fast division or exact fallback
  s.n++;
  if (!fast) s.fallback++;
  if (f2bits(got) != f2bits(want) || (fast && f2bits(q) != f2bits(want))) {
    if (s.bad < 5) printf("# %s mismatch ratio=%a got=%a exact=%a\n", s.name, ratio, got, want);
    s.bad++;
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 100000;
  rng_state = argc > 2 ? strtoull(argv[2], 0, 10) : 88172645463325252ULL;
  Stat rex{"rrec_exhaustive"}, rlg{"rrec_lognormal"}, rwd{"rrec_wide"}, res{"resid"}, src{"src"},
      xre{"xhi_realistic"}, xwd{"xhi_wide"};
  {
    const Consts c(7.0, 300.0, 512);
    if (!c.rf.ok || !c.pf_resid.ok) return 2;
    for (uint32_t b = f2bits(0.5f); b < f2bits(2.0f); ++b) check_rrec(rex, c, bits2f(b));
  }
  const double zs[6] = {5.0, 7.0, 8.5, 11.0, 15.0, 20.0};
  const double Ls[4] = {300.0, 106.5, 50.0, 1000.0};
  const int Ns[4] = {512, 600, 128, 1200};
  for (double z : zs)
    for (int bx = 0; bx < 4; ++bx) {
      const Consts c(z, Ls[bx], Ns[bx]);
      if (!c.rf.ok || !c.pf_resid.ok) return 2;
      // the source products: SFRD (dx^3 Qion(z), Qion as user_functions.c) and the
      // halo-branch ratio (dx_s / dx_h)^3
      const double dx = Ls[bx] / Ns[bx];
      const sd_t sfrd[4] = {d2bits(dx), d2bits(dx), d2bits(dx), d2bits(std::pow(10.0, 2.05707274e-02 * z + 5.29944413e+01) / 1.e+45)};
      const sd_t rion[1] = {d2bits(std::pow(dx / (Ls[bx] / (2 * Ns[bx])), 3))};
      const ProdFast ps = prod_fast_prepare(sfrd, 4), pr = prod_fast_prepare(rion, 1);
      if (!ps.ok || !pr.ok) return 2;
      for (long i = 0; i < n; ++i) {
        // lognormal 1 + d, sigma 1.5 (Box-Muller)
        const double gs = std::sqrt(-2.0 * std::log(1.0 - rnd_unit())) * std::cos(6.283185307179586 * rnd_unit());
        const float d = (float)(std::exp(1.5 * gs) - 1.0);
        const sd_t one_d = sd_add(0x3FF0000000000000ULL, sd_from_float(d));
        check_rrec(rlg, c, sd_to_float(one_d));
        check_rrec(rwd, c, rnd_float_exp(-60, 60));
        check_prod(res, one_d, c.pf_resid, c.resid, 3);
        // the residual fraction's argument as the prologue rounds it, then XHI
        const float fr = sd_to_float(sd_mul(sd_mul(sd_mul(one_d, c.resid[0]), c.resid[1]), c.resid[2]));
        check_xhi(xre, fr);
        check_xhi(xwd, rnd_float_exp(-40, 20));
        const float s = (i % 16 == 0) ? 0.0f : rnd_float_exp(-100, 60);
        check_prod(src, sd_from_float(s), ps, sfrd, 4);
        check_prod(src, sd_from_float(s), pr, rion, 1);
      }
    }
  for (const Stat* s : {&rex, &rlg, &rwd, &res, &src, &xre, &xwd})
    printf("%s %ld %ld %ld\n", s->name, s->n, s->bad, s->fallback);
  return 0;
}
