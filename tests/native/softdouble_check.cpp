// Host-side check of softdouble.h against the CPU's native double unit.
// Usage: softdouble_check <n_random> <seed>
// Prints one line per operation: name, cases, mismatches, max |ulp diff|.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "softdouble.h"

static double bits2d(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
static uint64_t d2bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
static uint32_t f2bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

static uint64_t rng_state;
static uint64_t rnd64() {
  rng_state ^= rng_state << 13; rng_state ^= rng_state >> 7; rng_state ^= rng_state << 17;
  return rng_state;
}
// random double with exponent in [emin, emax], random sign if sgn
static double rnd_double(int emin, int emax, bool sgn) {
  uint64_t fr = rnd64() & 0xFFFFFFFFFFFFFULL;
  int e = emin + (int)(rnd64() % (uint64_t)(emax - emin + 1));
  uint64_t s = sgn ? (rnd64() & 1) << 63 : 0;
  return bits2d(s | ((uint64_t)(e + 1023) << 52) | fr);
}

struct Stat { const char* name; long n = 0, bad = 0; long maxulp = 0; };
static void acc(Stat& s, uint64_t got, uint64_t want) {
  s.n++;
  if (got != want) {
    s.bad++;
    long d = (long)(got > want ? got - want : want - got);
    if (d > s.maxulp) s.maxulp = d;
  }
}

int main(int argc, char** argv) {
  long n = argc > 1 ? atol(argv[1]) : 1000000;
  rng_state = argc > 2 ? strtoull(argv[2], 0, 10) : 88172645463325252ULL;
  Stat sa{"add"}, ss{"sub"}, sm{"mul"}, sdv{"div"}, sdc{"div_c"}, sq{"sqrt"}, sqf{"sqrt_fast"}, sf{"to_float"},
      sff{"from_float"}, sp{"pow"}, sp4{"pow4"}, sp4x{"pow4_exact"}, spf{"pow_then_float"}, se{"exp"}, sp3{"pow3"};
  for (long i = 0; i < n; i++) {
    double a = rnd_double(-40, 40, true), b = rnd_double(-40, 40, true);
    if (i % 4 == 1) b = rnd_double(-2, 2, true) + a;  // near-cancellation cases
    if (i % 4 == 2) { uint64_t u = d2bits(a) ^ (rnd64() & 0xFF); b = -bits2d(u); }
    acc(sa, sd_add(d2bits(a), d2bits(b)), d2bits(a + b));
    acc(ss, sd_sub(d2bits(a), d2bits(b)), d2bits(a - b));
    acc(sm, sd_mul(d2bits(a), d2bits(b)), d2bits(a * b));
    acc(sdv, sd_div(d2bits(a), d2bits(b)), d2bits(a / b));
    acc(sdc, sd_div_c(d2bits(a), sd_divc_prepare(d2bits(b))), d2bits(a / b));
    {  // float numerators (the smoothed boxes) over a few fixed divisors
      float fa; uint32_t fb2 = (uint32_t)rnd64() & 0x7FFFFFFFu; std::memcpy(&fa, &fb2, 4);
      const double dvs[4] = {std::pow(0.0875, 3.0), std::pow(150.0 * 0.7 / 1200, 3.0), 27.0, 1.0 / 3.0};
      const double dv = dvs[i & 3];
      if (std::isfinite(fa) && fa != 0.0f && std::fabs(fa) >= 1.17549435e-38f)
        acc(sdc, sd_div_c(sd_from_float(fa), sd_divc_prepare(d2bits(dv))), d2bits((double)fa / dv));
    }
    double pa = std::fabs(a);
    acc(sq, sd_sqrt(d2bits(pa)), d2bits(std::sqrt(pa)));
    acc(sqf, sd_sqrt_fast(d2bits(pa)), d2bits(std::sqrt(pa)));
    {  // perfect squares and their neighbours
      const double r = (double)((rnd64() >> 38) | 1), sqv = r * r;
      for (int dd = -1; dd <= 1; ++dd) {
        const double v = bits2d(d2bits(sqv) + dd);
        acc(sqf, sd_sqrt_fast(d2bits(v)), d2bits(std::sqrt(v)));
      }
    }
    double fsrc = rnd_double(-150, 130, true);
    sf.n++;
    if (f2bits(sd_to_float(d2bits(fsrc))) != f2bits((float)fsrc)) sf.bad++;
    float ff; uint32_t fb = (uint32_t)rnd64(); std::memcpy(&ff, &fb, 4);
    if (std::isfinite(ff)) acc(sff, sd_from_float(ff), d2bits((double)ff));
    // pow over the prologue's domain: x in [2^-30, 2^30], y = 0.81722878 or 4
    double x = rnd_double(-30, 30, false);
    double y = 0.81722878;
    acc(sp, sd_pow(d2bits(x), d2bits(y)), d2bits(std::pow(x, y)));
    double x4 = rnd_double(-12, 0, false);
    acc(sp4, sd_pow(d2bits(x4), d2bits(4.0)), d2bits(std::pow(x4, 4.0)));
    {  // x^4 by exact squaring equals the correctly rounded sd_pow(x, 4)
      const double xq = (i & 1) ? x4 : rnd_double(-60, 60, false);
      acc(sp4x, sd_pow4(d2bits(xq)), sd_pow(d2bits(xq), d2bits(4.0)));
    }
    double xe = -rnd_double(-20, 9, false) * 0.68;  // exp over (-696, 0): normal results
    acc(se, sd_exp(d2bits(xe)), d2bits(std::exp(xe)));
    double x3 = rnd_double(-8, 8, false);
    acc(sp3, sd_pow(d2bits(x3), d2bits(3.0)), d2bits(std::pow(x3, 3.0)));
    spf.n++;
    if (f2bits(sd_to_float(sd_pow(d2bits(x), d2bits(y)))) != f2bits((float)std::pow(x, y))) spf.bad++;
  }
  Stat* all[] = {&sa, &ss, &sm, &sdv, &sdc, &sq, &sqf, &sf, &sff, &sp, &sp4, &sp4x, &spf, &se, &sp3};
  for (Stat* s : all) printf("%s %ld %ld %ld\n", s->name, s->n, s->bad, s->maxulp);
  return 0;
}
