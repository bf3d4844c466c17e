// Host-side check of sg_dmul.h (the subgrid draw products) against the CPU's
// native double multiply: chains of uniforms x 2^-32 from a fixed seed.
// Usage: dmul_check <n_chains> <seed>; prints "cases mismatches".
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "sg_dmul.h"

using namespace sf21;

static uint64_t st;
static uint64_t rnd64() {
  st ^= st << 13;
  st ^= st >> 7;
  st ^= st << 17;
  return st;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  st = argc > 2 ? strtoull(argv[2], nullptr, 10) : 88172645463325252ULL;
  long cases = 0, bad = 0;
  for (long c = 0; c < n; ++c) {
    // a chain of up to 12 factors; small x now and then (few significant bits)
    uint32_t x = (uint32_t)rnd64();
    if ((c & 7) == 0) x >>= (rnd64() % 31);
    if (!x) x = 1;
    double prod = 1.0 * (x / 4294967296.0);
    DMant d = dm_from_u32(x);
    uint64_t pb;
    std::memcpy(&pb, &prod, 8);
    cases++;
    if (dm_to_bits(d) != pb) bad++;
    for (int k = 0; k < 12 && prod > 1e-250; ++k) {
      uint32_t y = (uint32_t)rnd64();
      if ((k & 3) == 0) y >>= (rnd64() % 31);
      if (!y) y = 1;
      prod *= y / 4294967296.0;
      d = dm_mul_u32(d, y);
      std::memcpy(&pb, &prod, 8);
      cases++;
      if (dm_to_bits(d) != pb) {
        if (bad < 5) fprintf(stderr, "mismatch %a vs bits %llx\n", prod, (unsigned long long)dm_to_bits(d));
        bad++;
      }
    }
  }
  printf("%ld %ld\n", cases, bad);
  return bad != 0;
}
