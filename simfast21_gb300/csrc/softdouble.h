// IEEE-754 binary64 arithmetic on 64-bit integers (round to nearest even).
//
// The HII prologue (get_HIIbubbles.c:216-225, 272-274, 281-288 and
// user_functions.c:58-106) computes every per-voxel quantity in double and
// rounds the result to float.  The GPU product path must not use FP64
// arithmetic, so these routines reproduce the same double operations bit for
// bit with integer instructions: add, sub, mul, div and sqrt are correctly
// rounded exactly like the hardware double unit of the reference's CPU.
// pow() is not an IEEE basic operation: sd_pow evaluates it in 64+ bit fixed
// point (error below 2^-59 relative) and rounds once, which returns the same
// double as a correctly rounded libm pow except in rare near-tie cases; the
// prologue rounds its results to float afterwards, which hides those cases.
//
// Domain handled: finite normal operands and zeros (the prologue never meets
// subnormal doubles, infinities or NaNs); sd_pow needs x >= 0 with a binary
// exponent in [-60, 60] and |y| < 64.  Outside it returns a quiet NaN so a
// violation is visible in the output instead of silently wrong.
//
// The same header compiles as host C++ (g++) so it can be checked against
// the CPU's native double unit without a GPU.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SD_HD __host__ __device__ __forceinline__
#else
#define SD_HD static inline
#endif

typedef uint64_t sd_t;
typedef unsigned __int128 sd_u128;
typedef __int128 sd_i128;

#define SD_SIGN (0x8000000000000000ULL)
#define SD_QNAN (0x7ff8000000000000ULL)

#include "pow_tables.h"

SD_HD int sd_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

SD_HD int sd_clz128(sd_u128 x) {
  uint64_t hi = (uint64_t)(x >> 64);
  if (hi) return sd_clz64(hi);
  return 64 + sd_clz64((uint64_t)x);
}

// Shift right with sticky bit (OR of the shifted-out bits) in bit 0.
SD_HD uint64_t sd_shr_sticky(uint64_t x, int s) {
  if (s <= 0) return x;
  if (s >= 64) return x != 0;
  return (x >> s) | ((x & ((1ULL << s) - 1)) != 0);
}

// Pack sign, unbiased exponent e and a significand m with its leading one at
// bit 62 (bits 61..10 fraction, 9..0 guard/sticky) into a rounded double.
// Results are assumed to stay in the normal range.
SD_HD sd_t sd_round_pack(uint64_t sign, int e, uint64_t m) {
  // m: leading one at bit 62.  Keep 53 bits (62..10), round on bits 9..0.
  uint64_t rest = m & 0x3FFULL;
  uint64_t q = m >> 10;  // 53 bits, leading one at bit 52
  if (rest > 0x200ULL || (rest == 0x200ULL && (q & 1))) {
    q += 1;
    if (q >> 53) {  // carry out: 1.111..1 + ulp = 10.0
      q >>= 1;
      e += 1;
    }
  }
  return sign | ((uint64_t)(e + 1023) << 52) | (q & 0xFFFFFFFFFFFFFULL);
}

SD_HD sd_t sd_from_float(float f) {
  union {
    float f;
    uint32_t u;
  } c;
  c.f = f;
  uint32_t u = c.u;
  uint64_t sign = (uint64_t)(u >> 31) << 63;
  uint32_t ex = (u >> 23) & 0xFF;
  uint32_t fr = u & 0x7FFFFF;
  if (ex == 0) {
    if (fr == 0) return sign;
    // subnormal float: normalise
    int sh = sd_clz64((uint64_t)fr) - 40;  // leading one to bit 23
    fr <<= sh;
    int e = -126 - sh;
    return sign | ((uint64_t)(e + 1023) << 52) | ((uint64_t)(fr & 0x7FFFFF) << 29);
  }
  if (ex == 0xFF) return sign | 0x7FF0000000000000ULL | ((uint64_t)fr << 29);
  return sign | ((uint64_t)(ex - 127 + 1023) << 52) | ((uint64_t)fr << 29);
}

SD_HD sd_t sd_from_int(int64_t v) {
  if (v == 0) return 0;
  uint64_t sign = v < 0 ? SD_SIGN : 0;
  uint64_t a = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
  int lz = sd_clz64(a);
  int e = 63 - lz;
  uint64_t m = a << lz;  // leading one at bit 63
  m = sd_shr_sticky(m, 1);
  return sd_round_pack(sign, e, m);
}

// Round a double to the nearest float (ties to even), with float subnormals.
SD_HD float sd_to_float(sd_t d) {
  uint32_t sign = (uint32_t)(d >> 63) << 31;
  int ex = (int)((d >> 52) & 0x7FF);
  uint64_t fr = d & 0xFFFFFFFFFFFFFULL;
  uint32_t out;
  if (ex == 0x7FF) {
    out = sign | 0x7F800000u | (fr ? 0x400000u : 0u);
  } else if (ex == 0) {
    out = sign;  // double subnormals underflow to zero in float
  } else {
    int e = ex - 1023;
    uint64_t m = fr | (1ULL << 52);  // 53-bit significand
    if (e > 127) {
      out = sign | 0x7F800000u;
    } else {
      int shift;      // bits to drop from the 53-bit significand
      int fe;         // float biased exponent for the result (0 = subnormal)
      if (e >= -126) {
        shift = 29;
        fe = e + 127;
      } else {
        shift = 29 + (-126 - e);
        fe = 0;
      }
      uint64_t q, rem, half;
      if (shift >= 64) {
        q = 0;
        rem = m;
        half = 0;  // m < 2^53 < half: always rounds down
        out = sign;
      } else {
        q = m >> shift;
        rem = m & ((1ULL << shift) - 1);
        half = 1ULL << (shift - 1);
        if (rem > half || (rem == half && (q & 1))) q += 1;
        if (fe == 0) {
          // subnormal (q may round up into the smallest normal: bit 23)
          out = sign | (uint32_t)q;
        } else {
          if (q >> 24) {
            q >>= 1;
            fe += 1;
          }
          if (fe >= 255)
            out = sign | 0x7F800000u;
          else
            out = sign | ((uint32_t)fe << 23) | ((uint32_t)q & 0x7FFFFFu);
        }
      }
    }
  }
  union {
    uint32_t u;
    float f;
  } c;
  c.u = out;
  return c.f;
}

SD_HD bool sd_is_zero(sd_t a) { return (a & ~SD_SIGN) == 0; }
SD_HD sd_t sd_neg(sd_t a) { return a ^ SD_SIGN; }

// Total order on finite values: a < b
SD_HD bool sd_lt(sd_t a, sd_t b) {
  if (sd_is_zero(a) && sd_is_zero(b)) return false;
  bool sa = a >> 63, sb = b >> 63;
  if (sa != sb) return sa;
  if (!sa) return a < b;
  return a > b;
}
SD_HD bool sd_gt(sd_t a, sd_t b) { return sd_lt(b, a); }
SD_HD bool sd_ge(sd_t a, sd_t b) { return !sd_lt(a, b); }

SD_HD sd_t sd_add(sd_t a, sd_t b) {
  if (sd_is_zero(a)) return sd_is_zero(b) ? (a & b) : b;
  if (sd_is_zero(b)) return a;
  int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  if (ea == 0x7FF || eb == 0x7FF || ea == 0 || eb == 0) return SD_QNAN;
  uint64_t sa = a & SD_SIGN, sb = b & SD_SIGN;
  // significands with the leading one at bit 61: value = m * 2^(e - 61)
  uint64_t ma = ((a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) << 9;
  uint64_t mb = ((b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) << 9;
  if (ea < eb || (ea == eb && ma < mb)) {  // make |a| >= |b|
    uint64_t t = ma; ma = mb; mb = t;
    int te = ea; ea = eb; eb = te;
    uint64_t ts = sa; sa = sb; sb = ts;
  }
  mb = sd_shr_sticky(mb, ea - eb);
  // sd_round_pack wants value = m * 2^(e - 62) with the leading one at 62
  int e = ea - 1023 + 1;
  uint64_t m;
  if (sa == sb) {
    m = ma + mb;  // < 2^63
    if (!(m >> 62)) {
      m <<= 1;
      e -= 1;
    }
  } else {
    m = ma - mb;
    if (m == 0) return 0;  // exact cancellation: +0 under round-to-nearest
    int sh = sd_clz64(m) - 1;  // bring the leading one to bit 62
    m <<= sh;
    e -= sh;
  }
  return sd_round_pack(sa, e, m);
}

SD_HD sd_t sd_sub(sd_t a, sd_t b) { return sd_add(a, sd_neg(b)); }

SD_HD sd_t sd_mul(sd_t a, sd_t b) {
  uint64_t sign = (a ^ b) & SD_SIGN;
  if (sd_is_zero(a) || sd_is_zero(b)) return sign;
  int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  if (ea == 0x7FF || eb == 0x7FF || ea == 0 || eb == 0) return SD_QNAN;
  uint64_t ma = (a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  uint64_t mb = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  sd_u128 p = (sd_u128)ma * mb;  // leading one at bit 104 or 105
  int e = (ea - 1023) + (eb - 1023);
  // bring leading one to bit 62 of a 64-bit word with sticky
  int lead = 127 - sd_clz128(p);  // 104 or 105
  int sh = lead - 62;
  uint64_t hi = (uint64_t)(p >> sh);
  uint64_t sticky = (p & (((sd_u128)1 << sh) - 1)) != 0;
  e += lead - 104;
  return sd_round_pack(sign, e, hi | sticky);
}

SD_HD sd_t sd_div(sd_t a, sd_t b) {
  uint64_t sign = (a ^ b) & SD_SIGN;
  if (sd_is_zero(b)) return SD_QNAN;
  if (sd_is_zero(a)) return sign;
  int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  if (ea == 0x7FF || eb == 0x7FF || ea == 0 || eb == 0) return SD_QNAN;
  uint64_t ma = (a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  uint64_t mb = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  int e = (ea - 1023) - (eb - 1023);
  if (ma < mb) {
    ma <<= 1;
    e -= 1;
  }
  // quotient ma/mb in [1, 2): produce 63 bits (leading one at bit 62)
  sd_u128 num = (sd_u128)ma << 62;
  uint64_t q = (uint64_t)(num / mb);
  uint64_t r = (uint64_t)(num - (sd_u128)q * mb);
  return sd_round_pack(sign, e, q | (r != 0));
}

// Division by an invariant divisor.  The 128/64-bit integer step of sd_div
// is done with a precomputed reciprocal, the method of N. Moeller and
// T. Granlund, "Improved division by invariant integers", IEEE Trans.
// Computers 60(2), 2011 (Algorithm 4): two multiplications and at most two
// corrections instead of a software 128-bit division.  Same results as
// sd_div (the quotient and its remainder are exact).
typedef struct {
  uint64_t d;     // divisor significand, leading one at bit 63
  uint64_t v;     // floor((2^128 - 1) / d) - 2^64
  uint64_t sign;  // divisor sign bit
  int eb;         // divisor's unbiased exponent
  int ok;         // 0: divisor zero, subnormal, infinite or NaN (results are NaN)
} sd_divc;

SD_HD sd_divc sd_divc_prepare(sd_t b) {
  sd_divc k;
  const int eb = (int)((b >> 52) & 0x7FF);
  k.ok = !(sd_is_zero(b) || eb == 0x7FF || eb == 0);
  const uint64_t mb = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  k.d = mb << 11;
  // (2^128 - 1) / d - 2^64 = ((2^64 - 1 - d) * 2^64 + 2^64 - 1) / d
  k.v = (uint64_t)((((sd_u128)(~k.d)) << 64 | (sd_u128)0xFFFFFFFFFFFFFFFFULL) / k.d);
  k.sign = b & SD_SIGN;
  k.eb = eb - 1023;
  return k;
}

SD_HD sd_t sd_div_c(sd_t a, const sd_divc k) {
  const uint64_t sign = (a & SD_SIGN) ^ k.sign;
  if (!k.ok) return SD_QNAN;
  if (sd_is_zero(a)) return sign;
  const int ea = (int)((a >> 52) & 0x7FF);
  if (ea == 0x7FF || ea == 0) return SD_QNAN;
  uint64_t ma = (a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const uint64_t mb = k.d >> 11;
  int e = (ea - 1023) - k.eb;
  if (ma < mb) {
    ma <<= 1;
    e -= 1;
  }
  // (ma << 62) / mb = ((ma << 62) << 11) / d: the two-word numerator is
  // u1 = ma << 9, u0 = 0, with u1 < d since ma < 2 mb
  const uint64_t u1 = ma << 9, u0 = 0;
  const sd_u128 p = (sd_u128)k.v * u1;
  uint64_t q0 = (uint64_t)p + u0;
  uint64_t q1 = (uint64_t)(p >> 64) + u1 + (q0 < u0 ? 1 : 0) + 1;
  uint64_t r = u0 - q1 * k.d;
  if (r > q0) {
    q1 -= 1;
    r += k.d;
  }
  if (r >= k.d) {
    q1 += 1;
    r -= k.d;
  }
  return sd_round_pack(sign, e, q1 | (r != 0));
}

SD_HD sd_t sd_sqrt(sd_t a) {
  if (sd_is_zero(a)) return a;
  if (a >> 63) return SD_QNAN;
  int ea = (int)((a >> 52) & 0x7FF);
  if (ea == 0x7FF || ea == 0) return SD_QNAN;
  uint64_t m = (a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  int e = ea - 1023;
  if (e & 1) {
    m <<= 1;
    e -= 1;
  }
  // sqrt(m * 2^-52) * 2^(e/2); want 63-bit root of m * 2^(124-52) = m << 72
  sd_u128 x = (sd_u128)m << 72;  // value in [2^124, 2^126)
  // integer sqrt, bit by bit
  sd_u128 res = 0, bit = (sd_u128)1 << 126;
  while (bit > x) bit >>= 2;
  while (bit != 0) {
    if (x >= res + bit) {
      x -= res + bit;
      res = (res >> 1) + bit;
    } else {
      res >>= 1;
    }
    bit >>= 2;
  }
  uint64_t r = (uint64_t)res;  // leading one at bit 62
  return sd_round_pack(0, e / 2, r | (x != 0));
}

// sqrt by a fixed-point reciprocal-square-root Newton iteration from a float
// seed, then an exact integer correction: the same result as the digit-by-
// digit sd_sqrt, without its 63 iterations on 128-bit values.
SD_HD uint64_t sd_mulhi64(uint64_t a, uint64_t b) { return (uint64_t)(((sd_u128)a * b) >> 64); }

SD_HD sd_t sd_sqrt_fast(sd_t a) {
  if (sd_is_zero(a)) return a;
  if (a >> 63) return SD_QNAN;
  int ea = (int)((a >> 52) & 0x7FF);
  if (ea == 0x7FF || ea == 0) return SD_QNAN;
  uint64_t m = (a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  int e = ea - 1023;
  if (e & 1) {
    m <<= 1;
    e -= 1;
  }
  // x = m << 72 in [2^124, 2^126); X = x / 2^124 = m / 2^52 in [1, 4), Q62: m << 10
  const uint64_t Xq = m << 10;
  // y = 1/sqrt(X) in Q63, seeded in float (~24 bits), three Newton steps
  // y <- y (3 - X y^2) / 2 (each roughly doubles the good bits, to the Q63 limit)
  const float Xf = (float)m * 2.220446049250313e-16f;  // m / 2^52
  const float yf = 1.0f / sqrtf(Xf);
  uint64_t y = yf >= 1.0f ? (1ULL << 63) : (uint64_t)(yf * 9.223372036854775808e18f);
  for (int it = 0; it < 3; ++it) {
    const uint64_t y2 = sd_mulhi64(y, y);              // y^2 in Q62 (y^2 <= 1)
    const uint64_t t = sd_mulhi64(Xq, y2);             // X y^2, Q60
    const uint64_t u = (3ULL << 60) - t;               // 3 - X y^2, Q60
    const uint64_t yn = sd_mulhi64(y, u) << 3;         // y u / 2, Q63
    y = yn;
  }
  // r = sqrt(x) = sqrt(X) 2^62 = X y 2^62: mulhi(Xq, y) = X y 2^61
  uint64_t r = sd_mulhi64(Xq, y) << 1;
  const sd_u128 x = (sd_u128)m << 72;
  // exact correction to floor(sqrt(x)): a few units at most; bounded, with
  // the digit-by-digit routine as the fallback
  int fix = 0;
  while ((sd_u128)r * r > x && fix < 64) {
    --r;
    ++fix;
  }
  while ((sd_u128)(r + 1) * (r + 1) <= x && fix < 64) {
    ++r;
    ++fix;
  }
  if (fix >= 64) return sd_sqrt(a);
  return sd_round_pack(0, e / 2, r | ((sd_u128)r * r != x));
}

// Exact multiplication by 2^k for normal results.
SD_HD sd_t sd_ldexp(sd_t a, int k) {
  if (sd_is_zero(a)) return a;
  return a + ((uint64_t)(int64_t)k << 52);
}

// ---- pow(x, y) for x >= 0 via fixed point log2 / exp2 --------------------
// (a * b) >> 124 for signed fixed-point values with |a|, |b| < 2^126 and a
// result below 2^127, computed with 62-bit limbs so that no partial product
// exceeds 128 bits.  Truncation error: a few units of 2^-124.
SD_HD sd_i128 sd_mulq124(sd_i128 a, sd_i128 b) {
  bool neg = (a < 0) != (b < 0);
  sd_u128 ua = a < 0 ? (sd_u128)(-a) : (sd_u128)a;
  sd_u128 ub = b < 0 ? (sd_u128)(-b) : (sd_u128)b;
  const sd_u128 mask62 = (((sd_u128)1) << 62) - 1;
  uint64_t a0 = (uint64_t)(ua & mask62), a1 = (uint64_t)(ua >> 62);
  uint64_t b0 = (uint64_t)(ub & mask62), b1 = (uint64_t)(ub >> 62);
  sd_u128 p11 = (sd_u128)a1 * b1;                     // weight 2^124
  sd_u128 p10 = (sd_u128)a1 * b0 + (sd_u128)a0 * b1;  // weight 2^62
  sd_u128 p00 = (sd_u128)a0 * b0;                     // weight 1
  sd_u128 r = p11 + (p10 >> 62) + (((p10 & mask62) + (p00 >> 62)) >> 62);
  return neg ? -(sd_i128)r : (sd_i128)r;
}

#define SD_Q124(hi, lo) ((sd_i128)((((sd_u128)(hi)) << 64) | (sd_u128)(lo)))

// log2(x) = e + log2(c_j) + ln(1 + t)/ln 2 with c_j = 2^62 / SD_POW_INV[j]
// (j = top 7 fraction bits of x) and t = m/c_j - 1 exactly, |t| <= 2^-8; the
// series for ln(1 + t) to t^9 leaves < 2^-83.  w = y log2(x) is kept in Q.96
// and 2^w = 2^n 2^(j2/128) e^u with u = r ln 2 < 2^-7.5 and e^u to u^10.
// Every constant is a Q.124 (or Q.96) fixed-point number, so the relative
// error of the result before the final rounding is far below 2^-80.
// log2(x) in Q.96 for a positive normal x with binary exponent in [-60, 60].
SD_HD sd_i128 sd_log2_q96(sd_t x) {
  const int ex = (int)((x >> 52) & 0x7FF) - 1023;
  const uint64_t M = (x & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const int j = (int)((M >> 45) & 127);
  // m/c_j = M * INV[j] / 2^114 (exact); t in Q.124
  const sd_u128 P = (sd_u128)M * SD_POW_INV[j];
  const sd_i128 T = (sd_i128)(P << 10) - (((sd_i128)1) << 124);
  sd_i128 acc = SD_Q124(SD_POW_RCP_HI[9], SD_POW_RCP_LO[9]);
  for (int k = 8; k >= 1; --k)
    acc = SD_Q124(SD_POW_RCP_HI[k], SD_POW_RCP_LO[k]) - sd_mulq124(T, acc);
  const sd_i128 lnp = sd_mulq124(T, acc);  // ln(1 + t), Q.124, |lnp| < 2^117
  sd_i128 l2 = sd_mulq124(lnp, SD_Q124(SD_POW_INV_LN2_HI, SD_POW_INV_LN2_LO)) >> 28;
  l2 += (sd_i128)(((sd_u128)SD_POW_L2C_HI[j] << 64) | SD_POW_L2C_LO[j]);
  l2 += ((sd_i128)ex) << 96;  // |l2| < 2^103
  return l2;
}

// 2^(y * l2) for a double y with binary exponent in [-60, 10] and l2 in Q.96
// (|l2| < 2^103), rounded once to double; 0 / inf outside the range.
SD_HD sd_t sd_exp2_mul(sd_t y, sd_i128 l2) {
  const int ey = (int)((y >> 52) & 0x7FF) - 1023;
  // w = y * l2 in Q.96, y = my * 2^(ey - 52)
  const uint64_t my = (y & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const bool wneg = ((y >> 63) != 0) != (l2 < 0);
  const sd_u128 ul2 = l2 < 0 ? (sd_u128)(-l2) : (sd_u128)l2;
  const uint64_t u0 = (uint64_t)ul2, u1 = (uint64_t)(ul2 >> 64);  // u1 < 2^39
  const sd_u128 q0 = (sd_u128)u0 * my;  // weight 1
  const sd_u128 q1 = (sd_u128)u1 * my;  // weight 2^64, < 2^92
  const int s = 52 - ey;                // >= 42
  sd_u128 w;                            // |w| in Q.96
  if (s <= 64)
    w = (q1 << (64 - s)) + (q0 >> s);
  else
    w = (q1 >> (s - 64)) + (s < 128 ? (q0 >> s) : 0);
  int64_t n = (int64_t)(w >> 96);
  sd_u128 f = w & ((((sd_u128)1) << 96) - 1);
  if (wneg) {
    if (f != 0) {
      n = -n - 1;
      f = (((sd_u128)1) << 96) - f;
    } else {
      n = -n;
    }
  }
  if (n > 1023) return 0x7FF0000000000000ULL;
  if (n < -1022) return 0;  // below the normal range (not met by the prologue)
  const int j2 = (int)(f >> 89);
  const sd_i128 r = (sd_i128)((f & ((((sd_u128)1) << 89) - 1)) << 28);  // Q.124, < 2^-7
  const sd_i128 u = sd_mulq124(r, SD_Q124(SD_POW_LN2_HI, SD_POW_LN2_LO));
  sd_i128 ex_u = SD_Q124(SD_POW_IFACT_HI[10], SD_POW_IFACT_LO[10]);
  for (int k = 9; k >= 0; --k)
    ex_u = SD_Q124(SD_POW_IFACT_HI[k], SD_POW_IFACT_LO[k]) + sd_mulq124(u, ex_u);
  // significand 2^(j2/128) e^u, Q.124, value in [1, 2.02)
  const sd_u128 mm =
      (sd_u128)sd_mulq124(SD_Q124(SD_POW_EXP2T_HI[j2], SD_POW_EXP2T_LO[j2]), ex_u);
  const int lead = (mm >> 125) ? 125 : 124;
  const int sh = lead - 62;
  const uint64_t m = (uint64_t)(mm >> sh) | ((mm & ((((sd_u128)1) << sh) - 1)) != 0);
  return sd_round_pack(0, (int)n + (lead - 124), m);
}

SD_HD sd_t sd_pow(sd_t x, sd_t y) {
  if (sd_is_zero(y)) return 0x3FF0000000000000ULL;
  if (sd_is_zero(x)) return (y >> 63) ? 0x7FF0000000000000ULL : 0;
  if (x >> 63) return SD_QNAN;
  const int ex = (int)((x >> 52) & 0x7FF) - 1023;
  const int ey = (int)((y >> 52) & 0x7FF) - 1023;
  if (ex < -60 || ex > 60 || ey > 5 || ey < -60) return SD_QNAN;
  return sd_exp2_mul(y, sd_log2_q96(x));
}

// x^4 for x > 0, correctly rounded (the same value as sd_pow(x, 4.0)): the
// 212-bit integer m^4 of the significand, rounded once.  Exponents outside
// [-60, 60] take sd_pow's path.
SD_HD sd_t sd_pow4(sd_t x) {
  if (sd_is_zero(x) || (x >> 63)) return sd_pow(x, 0x4010000000000000ULL);
  const int ex = (int)((x >> 52) & 0x7FF) - 1023;
  if (ex < -60 || ex > 60) return sd_pow(x, 0x4010000000000000ULL);
  const uint64_t m = (x & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const sd_u128 m2 = (sd_u128)m * m;  // < 2^106
  const uint64_t h = (uint64_t)(m2 >> 64), l = (uint64_t)m2;
  // m^4 = h^2 2^128 + 2 h l 2^64 + l^2 as four 64-bit words w3..w0
  const sd_u128 ll = (sd_u128)l * l, hl = (sd_u128)h * l, hh = (sd_u128)h * h;
  uint64_t w0 = (uint64_t)ll;
  sd_u128 t = (ll >> 64) + ((sd_u128)(uint64_t)hl << 1);
  uint64_t w1 = (uint64_t)t;
  t = (t >> 64) + ((hl >> 64) << 1) + ((uint64_t)hl >> 63) + (uint64_t)hh;
  uint64_t w2 = (uint64_t)t;
  uint64_t w3 = (uint64_t)(t >> 64) + (uint64_t)(hh >> 64);
  // leading one at bit L of the 256-bit number (208 <= L <= 211): w3 holds bits 192..255
  const int L = 255 - sd_clz64(w3);
  // 63 bits from bit L down (leading one at bit 62), sticky for the rest
  const int sh = L - 62 - 128;  // shift of (w3:w2) right, 18..21
  const uint64_t top = (w3 << (64 - sh)) | (w2 >> sh);
  const uint64_t sticky = ((w2 & ((1ULL << sh) - 1)) | w1 | w0) != 0;
  return sd_round_pack(0, 4 * ex + (L - 208), top | sticky);
}

// exp(x) = 2^(x log2 e), correctly rounded for |x| < 2048 with a normal
// result; results below the double normal range return 0 (they round to 0 in
// float, which is all the stage keeps).
SD_HD sd_t sd_exp(sd_t x) {
  if (sd_is_zero(x)) return 0x3FF0000000000000ULL;
  const int ex = (int)((x >> 52) & 0x7FF) - 1023;
  if (ex < -60) return 0x3FF0000000000000ULL;  // |x| < 2^-60: exp(x) rounds to 1
  if (ex > 10) return (x >> 63) ? 0 : 0x7FF0000000000000ULL;
  const sd_i128 log2e = (sd_i128)(((sd_u128)SD_EXP_LOG2E_HI << 64) | SD_EXP_LOG2E_LO);  // Q.96
  return sd_exp2_mul(x, log2e);
}
