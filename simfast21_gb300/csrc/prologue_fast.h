// Fast paths for the HII prologue's per-voxel double chains, each returning
// the float that the exact chain would return (get_HIIbubbles.c:216-225,
// 272-274; user_functions.c:58-65, 101-106).
//
// The reference computes each per-voxel quantity as a chain of double
// operations and keeps only the result rounded to float.  softdouble.h
// reproduces every double operation bit for bit in integer arithmetic.  That
// is exact but long: a 124-bit fixed-point pow, a 212-bit fourth power, and
// 128/64-bit integer divisions.  The fast paths here evaluate the chain's
// real-number value F in 64-bit fixed point, with a proven relative error
// bound e_F.  The exact chain's double result D lies within a bound e_D of the
// same real number; each function states both bounds.  With e_D + e_F below
// 2^-48 and F further than 2^-46 (relative) from every float rounding
// midpoint, D and F round to the same float, which is returned
// (pf_round_guard).  Otherwise, or when an operand is outside the path's
// range, the function returns false and the caller evaluates the exact
// chain.  Float midpoints are 2^-23 apart (relative), so the guard band
// catches about one input in 2^21.
//
// Host and device compile the same code, so the CPU tests can compare every
// fast path with its exact chain on any number of inputs.
#pragma once
#include "softdouble.h"

// ---- shared pieces ----------------------------------------------------------

// floor(a b / 2^62) for signed Q.62 values whose product stays below 2^125.
SD_HD int64_t pf_mulq62(int64_t a, int64_t b) { return (int64_t)(((sd_i128)a * b) >> 62); }

// Product of two significands with bit 63 set, normalised so that bit 63 is
// set again.  *e gains the product's binary exponent change.  Relative
// truncation error below 2^-62.
SD_HD uint64_t pf_mulnorm(uint64_t a, uint64_t b, int* e) {
  const sd_u128 p = (sd_u128)a * b;  // in [2^126, 2^128)
  if (p >> 127) return (uint64_t)(p >> 64);
  *e -= 1;
  return (uint64_t)(p >> 63);
}

// 1 / S for S in Q.62, [1, 2): two Newton steps from a float reciprocal
// (relative error 2^-23 -> 2^-46 -> below 3 units of 2^-62).  Newton's
// iterates for the reciprocal approach 1/S from below, up to the
// truncations, so the result is in (2^61, 2^62 + 1].
SD_HD int64_t pf_recip_q62(uint64_t S) {
  const float sf = (float)(S >> 32) * (1.0f / 1073741824.0f);  // S 2^-62 in float
  const float yf = 1.0f / sf;
  int64_t Y = (int64_t)(yf * 4611686018427387904.0f);           // Q.62
  const int64_t S62 = (int64_t)S;
  for (int it = 0; it < 2; ++it)  // 2 - S Y in Q.62 (2 = 2^63 as unsigned)
    Y = pf_mulq62(Y, (int64_t)((1ULL << 63) - (uint64_t)pf_mulq62(S62, Y)));
  return Y;
}

SD_HD float pf_bits_float(uint32_t u) {
  union {
    uint32_t u;
    float f;
  } c;
  c.u = u;
  return c.f;
}

// Round F = Fm 2^(eF - 64) (bit 63 of Fm set) to float, with sign bit `sign`
// (bit 31).  Returns false when F lies within 2^18 units of Fm (relative
// 2^-46) of a float rounding midpoint, or when the float would not be normal.
SD_HD bool pf_round_guard(uint64_t Fm, int eF, uint32_t sign, float* out) {
  const uint64_t rem = Fm & ((1ULL << 40) - 1);  // the dropped bits; midpoint 2^39
  const uint64_t half = 1ULL << 39;
  const uint64_t dist = rem > half ? rem - half : half - rem;
  if (dist <= (1ULL << 18)) return false;
  uint32_t sig = (uint32_t)(Fm >> 40) + (rem > half ? 1u : 0u);
  int E = eF - 1;  // F = (Fm / 2^63) 2^(eF - 1)
  if (sig >> 24) {
    sig >>= 1;
    E += 1;
  }
  if (E < -126 || E > 127) return false;
  *out = pf_bits_float(sign | ((uint32_t)(E + 127) << 23) | (sig & 0x7FFFFFu));
  return true;
}

// ---- products by constants: (..((x k0) k1)..) k[n-1] -----------------------
// The source conversion (:272-274, or :258 for the halo branch) and the
// residual-fraction argument (1 + d) 1.881e-7 (1+z)^3 G_H(z) (:220).
// e_D: n roundings, n u (u = 2^-53, n <= 6).  e_F: the constants' product
// kept to 64 bits (n - 1 truncations) and the final product, below 2^-60.
struct ProdFast {
  uint64_t km;     // K = k0 k1 .. = km 2^(kx - 64), bit 63 of km set
  int kx;
  int emin, emax;  // range of the partial products' exponents relative to x's
  int ok;          // 0: constants outside the path's range (exact chain always)
};

SD_HD bool prod_fast(sd_t x, const ProdFast& k, float* out) {
  if (!k.ok) return false;
  const uint32_t sign = (uint32_t)(x >> 63) << 31;
  const int ex = (int)((x >> 52) & 0x7FF);
  if (ex == 0x7FF) return false;
  if (ex == 0) {
    if ((x << 1) != 0) return false;  // subnormal
    *out = pf_bits_float(sign);       // +-0 k = +-0 for positive constants
    return true;
  }
  const int e = ex - 1023;
  // every partial product stays a normal double, as the n u bound assumes
  if (e + k.emin < -1000 || e + k.emax > 1000) return false;
  const uint64_t mx = ((x & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) << 11;  // x = mx 2^(e + 1 - 64)
  int eF = e + 1 + k.kx;
  const uint64_t Fm = pf_mulnorm(mx, k.km, &eF);
  return pf_round_guard(Fm, eF, sign, out);
}

// ---- one division: a / b rounded to double, then to float --------------------
// XHI's last step (user_functions.c:105).  e_D: u/2.  e_F: the reciprocal
// (2^-59.4) and the product (2^-62), below 2^-59.
SD_HD bool div_fast(sd_t a, sd_t b, float* out) {
  const uint32_t sign = (uint32_t)((a ^ b) >> 63) << 31;
  const int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  if (eb == 0 || eb == 0x7FF || ea == 0x7FF) return false;
  if (ea == 0) {
    if ((a << 1) != 0) return false;
    *out = pf_bits_float(sign);
    return true;
  }
  const uint64_t ma = ((a & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) << 11;  // a = ma 2^(ea - 1023 + 1 - 64)
  const uint64_t S = ((b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) << 10;   // b's significand, Q.62
  const int64_t Y = pf_recip_q62(S);
  if (Y <= 0) return false;
  const int lz = sd_clz64((uint64_t)Y);
  // 1 / b = (Y << lz) 2^(2 - lz - 64) 2^-(eb - 1023)
  int eF = (ea - 1023 + 1) + (2 - lz) - (eb - 1023);
  const uint64_t Fm = pf_mulnorm(ma, (uint64_t)Y << lz, &eF);
  return pf_round_guard(Fm, eF, sign, out);
}

// ---- the recombination rate -------------------------------------------------
// density_map[i] = (float)Rrec((float)(1 + d), z) (:222, user_functions.c:58-65):
//   Rrec = rec1 * pow(rec2 / (1 + rec2), 4) * dvv / v_norm,  rec2 = pow(od / r2, r3).
// Real value: V = C (1 + 2^-w)^-4, w = r3 (log2 od - log2 r2), C = rec1 dvv / v_norm.
// e_D: od / r2 adds u, amplified by r3 < 1.  pow adds u plus at most 2^-59.
// 1 + rec2 and the division add 2u.  The fourth power multiplies that sum
// (3.9 u) by 4 and adds u.  The two products and the division by v_norm add
// 3u more: 19.4 u < 2^-48.6.  e_F: below 2^-56 (each step's bound is written
// at the step).
struct RrecFast {
  int64_t l2r2;  // log2(r2), Q.62
  uint64_t r3;   // r3, Q.63 (2^-11 <= r3 < 1)
  uint64_t cm;   // C = cm 2^(cx - 64), bit 63 of cm set
  int cx;
  int ok;        // 0: constants outside the path's range (exact chain always)
};

// The exact chain, operation by operation as user_functions.c:58-65.
SD_HD sd_t rrec_exact(float od, const sd_divc& r2c, sd_t r3, sd_t rec1, sd_t dvv, const sd_divc& v_normc) {
  const sd_t rec2 = sd_pow(sd_div_c(sd_from_float(od), r2c), r3);
  const sd_t q = sd_div(rec2, sd_add(0x3FF0000000000000ULL, rec2));
  const sd_t rec3 = sd_pow4(q);  // pow(.., 4.): correctly rounded like sd_pow
  return sd_div_c(sd_mul(sd_mul(rec1, rec3), dvv), v_normc);
}

// Float value of Rrec(od) in *out and true, or false (guard band, od outside
// [2^-60, 2^61), a result outside the normal float range, or constants out of
// range): the caller then uses rrec_exact.
SD_HD bool rrec_fast(float od, const RrecFast& k, float* out) {
  union {
    float f;
    uint32_t u;
  } cv;
  cv.f = od;
  const uint32_t fb = cv.u;
  const int eo = (int)((fb >> 23) & 255);
  if (!k.ok || (fb >> 31) || eo == 0 || eo == 255) return false;
  const int e = eo - 127;
  if (e < -60 || e > 60) return false;

  // log2(od) = e + log2(c_j) + ln(1 + t) / ln 2, c_j = 2^62 / SD_POW_INV[j]
  // (the table of sd_pow, j = top 7 fraction bits), t = m / c_j - 1 with
  // |t| <= 2^-8.  t is taken exactly from the 86-bit product and truncated to
  // Q.62.  The series to t^7 leaves |t|^8 / 8 < 2^-67.  The Horner steps,
  // 1/ln 2 and the two tables add at most 6 units of 2^-62.
  const uint64_t mo = (fb & 0x7FFFFFu) | 0x800000u;  // m 2^23
  const int j = (int)((mo >> 16) & 127);
  const sd_u128 P = (sd_u128)mo * SD_POW_INV[j];     // (m / c_j) 2^85
  const int64_t T = (int64_t)(((sd_i128)P - ((sd_i128)1 << 85)) >> 23);
  const int64_t Q1 = (int64_t)1 << 62;
  int64_t acc = Q1 / 7;
  acc = -(Q1 / 6) + pf_mulq62(T, acc);
  acc = Q1 / 5 + pf_mulq62(T, acc);
  acc = -(Q1 / 4) + pf_mulq62(T, acc);
  acc = Q1 / 3 + pf_mulq62(T, acc);
  acc = -(Q1 / 2) + pf_mulq62(T, acc);
  acc = Q1 + pf_mulq62(T, acc);
  const int64_t lnp = pf_mulq62(T, acc);  // ln(1 + t)
  const int64_t inv_ln2 = (int64_t)((SD_POW_INV_LN2_HI << 2) | (SD_POW_INV_LN2_LO >> 62));
  const int64_t l2c = (int64_t)((SD_POW_L2C_HI[j] << 30) | (SD_POW_L2C_LO[j] >> 34));
  const int64_t dfrac = l2c + pf_mulq62(lnp, inv_ln2) - k.l2r2;  // |dfrac| < 2

  // w = r3 (e + dfrac) in Q.63; error at most r3 6 + 1/2 units of 2^-62, under
  // 2^-59.6.  v = -w = nv + f with f in [0, 1).
  const sd_i128 W = (sd_i128)k.r3 * e + (((sd_i128)k.r3 * dfrac) >> 62);
  const sd_i128 V = -W;
  const int nv = (int)(V >> 63);
  const uint64_t f = (uint64_t)(V - (sd_i128)nv * ((sd_i128)1 << 63));  // Q.63 (nv may be negative)

  // 2^f = 2^(j2/128) e^x, x = (f - j2/128) ln 2 < 2^-7.5, series to x^6
  // (remainder < 2^-65).  U in Q.62, [1, 2); relative error (the error of w
  // included) below 2^-59.2.
  const int j2 = (int)(f >> 56);
  const int64_t ln2 = (int64_t)((SD_POW_LN2_HI << 2) | (SD_POW_LN2_LO >> 62));
  const int64_t X = pf_mulq62((int64_t)((f & ((1ULL << 56) - 1)) >> 1), ln2);
  int64_t ex = Q1 / 720;
  ex = Q1 / 120 + pf_mulq62(X, ex);
  ex = Q1 / 24 + pf_mulq62(X, ex);
  ex = Q1 / 6 + pf_mulq62(X, ex);
  ex = Q1 / 2 + pf_mulq62(X, ex);
  ex = Q1 + pf_mulq62(X, ex);
  ex = Q1 + pf_mulq62(X, ex);
  const int64_t e2t = (int64_t)((SD_POW_EXP2T_HI[j2] << 2) | (SD_POW_EXP2T_LO[j2] >> 62));
  const uint64_t U = (uint64_t)pf_mulq62(e2t, ex);

  // s = 1 + 2^-w = 1 + U 2^nv = S 2^es, S in Q.62, [1, 2); two truncations.
  uint64_t S;
  int es;
  if (nv >= 0) {
    S = U + (nv < 63 ? (1ULL << 62) >> nv : 0);
    es = nv;
  } else {
    S = (1ULL << 62) + (nv > -64 ? U >> (-nv) : 0);
    es = 0;
  }
  if (S >> 63) {
    S >>= 1;
    es += 1;
  }

  // y = 1 / S (3 units of 2^-62).  F = C y^4 2^(-4 es): three normalised
  // products (relative error < 2^-62 each).  Relative error of F: 4 x 2^-58.5
  // (s and y) plus the products and C, below 2^-56.
  const int64_t Y = pf_recip_q62(S);
  if (Y <= 0) return false;
  const int lz = sd_clz64((uint64_t)Y);
  const uint64_t ym = (uint64_t)Y << lz;  // y = ym 2^(2 - lz - 64)
  int e2 = 2 * (2 - lz);
  const uint64_t y2 = pf_mulnorm(ym, ym, &e2);
  int e4 = 2 * e2;
  const uint64_t y4 = pf_mulnorm(y2, y2, &e4);
  int eF = e4 + k.cx - 4 * es;
  const uint64_t Fm = pf_mulnorm(y4, k.cm, &eF);  // F = Fm 2^(eF - 64)
  return pf_round_guard(Fm, eF, 0u, out);
}

// ---- the residual neutral fraction -----------------------------------------
// XHI(ratio), user_functions.c:101-106, operation by operation in double.
SD_HD sd_t xhi_exact(sd_t r) {
  if (sd_is_zero(r)) return 0;
  const sd_t two_r = sd_ldexp(r, 1);                        // 2.*ratio (exact)
  const sd_t b = sd_add(two_r, 0x3FF0000000000000ULL);      // 2.*ratio + 1.
  const sd_t c = sd_mul(b, b);                              // (..)*(..)
  const sd_t e = sd_mul(sd_ldexp(r, 2), r);                 // 4.*ratio*ratio
  const sd_t g = sd_sqrt_fast(sd_sub(c, e));
  const sd_t num = sd_sub(b, g);                            // 2.*ratio + 1. - sqrt(..)
  return sd_div(num, two_r);                                // /(2.*ratio)
}

// (float)XHI(ratio).  The subtraction 2 ratio + 1 - sqrt(..) cancels most
// digits for small ratios, so every step before it stays exact; only the
// last division takes the fast path (div_fast).
SD_HD float xhi_float(float ratio) {
  const sd_t r = sd_from_float(ratio);
  if (sd_is_zero(r)) return 0.0f;
  const sd_t two_r = sd_ldexp(r, 1);
  const sd_t b = sd_add(two_r, 0x3FF0000000000000ULL);
  const sd_t c = sd_mul(b, b);
  const sd_t e = sd_mul(sd_ldexp(r, 2), r);
  const sd_t g = sd_sqrt_fast(sd_sub(c, e));
  const sd_t num = sd_sub(b, g);
  float x;
  if (!div_fast(num, two_r, &x)) x = sd_to_float(sd_div(num, two_r));
  return x;
}

// ---- host preparation of the constants (host code; visible to both nvcc passes) ---------------------------------------
static inline bool pf_normal_pos(sd_t x) {
  const int ex = (int)((x >> 52) & 0x7FF);
  return !(x >> 63) && ex != 0 && ex != 0x7FF;
}

// K = k0 k1 .. k[n-1] for positive normal doubles, kept to 64 bits after each
// product (truncation below 2^-63 per product).
static inline ProdFast prod_fast_prepare(const sd_t* ks, int n) {
  ProdFast k = {};
  if (n < 1 || n > 6) return k;
  uint64_t m = 1ULL << 63;
  int x = 1;  // value 1 = 2^63 2^(1 - 64)
  int pe = 0;
  k.emin = k.emax = 0;
  for (int i = 0; i < n; ++i) {
    if (!pf_normal_pos(ks[i])) return k;
    const int ei = (int)((ks[i] >> 52) & 0x7FF) - 1023;
    const uint64_t mi = ((ks[i] & 0xFFFFFFFFFFFFFULL) | (1ULL << 52)) << 11;
    x += ei + 1;
    m = pf_mulnorm(m, mi, &x);
    pe += ei;  // the i + 1 significands' product adds 0 .. i + 1 more
    if (pe < k.emin) k.emin = pe;
    if (pe + i + 1 > k.emax) k.emax = pe + i + 1;
  }
  k.km = m;
  k.kx = x;
  k.ok = 1;
  return k;
}

// log2 r2 from sd_pow's own fixed-point logarithm (error far below 2^-62);
// C from the exact 106-bit product rec1 dvv divided by v_norm in 128-bit
// integers (truncation below 2^-62 relative).
static inline RrecFast rrec_fast_prepare(sd_t rec1, sd_t dvv, sd_t v_norm, sd_t r2, sd_t r3) {
  RrecFast k = {};
  if (!pf_normal_pos(rec1) || !pf_normal_pos(dvv) || !pf_normal_pos(v_norm) || !pf_normal_pos(r2) ||
      !pf_normal_pos(r3))
    return k;
  const int e3 = (int)((r3 >> 52) & 0x7FF) - 1023;
  const int e2 = (int)((r2 >> 52) & 0x7FF) - 1023;
  if (e3 > -1 || e3 < -11 || e2 < -60 || e2 > 60) return k;
  const uint64_t m3 = (r3 & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  k.r3 = m3 << (11 + e3);  // r3 = m3 2^(e3 - 52) in Q.63
  k.l2r2 = (int64_t)(sd_log2_q96(r2) >> 34);
  const uint64_t ma = (rec1 & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const uint64_t mb = (dvv & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const uint64_t mv = (v_norm & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  const int ea = (int)((rec1 >> 52) & 0x7FF) - 1023;
  const int eb = (int)((dvv >> 52) & 0x7FF) - 1023;
  const int ev = (int)((v_norm >> 52) & 0x7FF) - 1023;
  // C = (ma mb / mv) 2^(ea + eb - ev - 52); q = floor(ma mb 2^22 / mv) in [2^73, 2^76)
  const sd_u128 q = (((sd_u128)ma * mb) << 22) / mv;
  const int lead = 127 - sd_clz128(q);
  k.cm = (uint64_t)(q >> (lead - 63));
  // C = q 2^(ea + eb - ev - 74) = (cm 2^-64) 2^(lead + 1 + ea + eb - ev - 74)
  k.cx = lead + 1 + ea + eb - ev - 74;
  k.ok = 1;
  return k;
}
