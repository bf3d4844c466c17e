// Exact IEEE double product of a positive normal double by a uniform
// u = x 2^-32 (x a nonzero 32-bit integer, exact in double), in integer
// arithmetic: the subgrid draw-length test multiplies such uniforms as the
// reference's `prod *= gsl_rng_uniform(r)` does (get_halos.c:353, the
// product-of-uniforms Poisson method), without the FP64 unit.
//
// A positive normal double is held as (m, e): value = m 2^(e - 52) with
// 2^52 <= m < 2^53.  The product m x has 53 to 85 bits; it is cut back to 53
// with round-to-nearest-even.  Results are assumed normal (the draw loop stops
// at a product <= exp(-mu) >= exp(-10) and every factor is >= 2^-32).
// Host and device (the host build is checked against the CPU's double unit).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SG_HD __host__ __device__ __forceinline__
#else
#define SG_HD static inline
#endif

namespace sf21 {

struct DMant {
  uint64_t m;
  int e;
};

SG_HD int dm_clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __clz(x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

SG_HD int dm_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

SG_HD uint64_t dm_mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

SG_HD DMant dm_from_u32(uint32_t x) {  // x 2^-32, x > 0
  const int lz = dm_clz32(x);
  DMant d;
  d.m = (uint64_t)x << (21 + lz);
  d.e = -1 - lz;
  return d;
}

// (m, e) from the bits of a positive normal double
SG_HD DMant dm_from_bits(uint64_t b) {
  DMant d;
  d.m = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  d.e = (int)((b >> 52) & 0x7FF) - 1023;
  return d;
}

SG_HD uint64_t dm_to_bits(DMant d) { return ((uint64_t)(d.e + 1023) << 52) | (d.m & 0xFFFFFFFFFFFFFULL); }

SG_HD DMant dm_mul_u32(DMant a, uint32_t x) {  // a * (x 2^-32), x > 0
  const uint64_t lo = a.m * (uint64_t)x;
  const uint64_t hi = dm_mulhi(a.m, (uint64_t)x);  // < 2^21
  const int nb = hi ? 128 - dm_clz64(hi) : 64 - dm_clz64(lo);  // 53..85
  const int sh = nb - 53;                                        // 0..32
  uint64_t q, rem, half;
  if (sh == 0) {
    q = lo;
    rem = 0;
    half = 1;
  } else {
    q = (lo >> sh) | (hi << (64 - sh));
    rem = lo & ((1ULL << sh) - 1);
    half = 1ULL << (sh - 1);
  }
  int e = a.e + sh - 32;
  if (rem > half || (rem == half && (q & 1))) {
    ++q;
    if (q >> 53) {
      q >>= 1;
      ++e;
    }
  }
  DMant r;
  r.m = q;
  r.e = e;
  return r;
}

SG_HD bool dm_le(DMant a, DMant b) { return a.e < b.e || (a.e == b.e && a.m <= b.m); }

}  // namespace sf21
