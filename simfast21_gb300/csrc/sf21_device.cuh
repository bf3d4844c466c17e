// Device-side data structures and helpers shared by the HII kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_line.cuh"

namespace sf21 {

// Max radii fused into one k-space pass (one spectrum read, K outputs).
constexpr int KMAX = 8;
// First-hit radius index sentinel: voxel was never a bubble centre.
constexpr uint8_t RC_NONE = 0xFF;

// One radius of a batch.
struct RadiusArg {
  float dkR;      // dk * R (k-space top-hat argument scale)
  int ridx;       // index of R in its parameter set's radius list
  float2* work;   // N^3 complex work buffer for this radius
};

struct Batch {    // radius indices r[k].ridx increase with k
  int K;          // radii in this batch (<= KMAX)
  int set;        // parameter set
  float zmul;     // ionisation-rate multiplier of the set (zeta)
  RadiusArg r[KMAX];
};

// Real-space top-hat window in k-space, W(x) = 3 (sin x - x cos x) / x^3
// (auxiliary.c:350-359).  Below x = 2 the Taylor series in x^2 (to x^14,
// truncation < 3e-11) avoids the cancellation of the closed form in float.
// Above, the closed form with sin/cos from the SFU (__sinf/__cosf: absolute
// error < 4e-7 on [-pi, pi]; a larger argument is reduced as x / 2 pi in
// single precision, which adds at most |x| 2^-24 to the angle) divided by x^3
// with the fast division (2 ulp).  With e = 4e-7 + 6e-8 x the error left in
// W is below 3 e (1 + x) / x^3 + 3e-7 |W| <= 6e-7 absolute for x >= 2
// (W(0) = 1), and falls as 1/x for large x: under the FP32 rounding of the
// transforms it feeds.
__device__ __forceinline__ float w_tophat(float x) {
  if (x < 2.0f) {
    const float y = x * x;
    float p = -1.3495220664131733e-13f;       // -1/7410154752000
    p = fmaf(p, y, 3.2118561710393668e-11f);  // 1/31135104000
    p = fmaf(p, y, -5.7812513436029994e-09f); // -1/172972800
    p = fmaf(p, y, 7.5156266505230805e-07f);  // 1/1330560
    p = fmaf(p, y, -6.6137566137566139e-05f); // -1/15120
    p = fmaf(p, y, 3.5714285714285713e-03f);  // 1/280
    p = fmaf(p, y, -0.1f);
    p = fmaf(p, y, 1.0f);
    return p;
  }
  const float s = __sinf(x), c = __cosf(x);
  return __fdividef(3.0f * fmaf(-x, c, s), x * x * x);  // 2 ulp; x^3 < 2^126 here
}

// Centre test (get_HIIbubbles.c:339-348) on a packed filtered value
// v = (rec_R, alpha * ion1_R), ion = ion1 * zeta:
//   centre <=> ion > 0 && (rec <= 0 || ion >= rec)
// (for floats h, d > 0, (double)h/d >= 1 <=> h >= d).  With zeta >= 0, ion > 0
// and rec <= 0 already give ion >= rec, so the test reduces to
// v.y > 0 && v.y * zeta >= v.x * alpha (alpha a power of two: exact scaling).
// The one difference, a NaN rec, does not arise from finite boxes.
// alpha <= 0 marks an ionisation box that is zero everywhere: no centre.
// Both products are rounded explicitly (__fmul_rn): left to the compiler,
// the comparison may become one fused multiply-add in one kernel and two
// rounded products in another, and the radius pipelines would then disagree
// on centres within an ulp of the threshold.
__device__ __forceinline__ bool is_centre(float2 v, float alpha, float zeta) {
  return (alpha > 0.0f) && (v.y > 0.0f) && (__fmul_rn(v.y, zeta) >= __fmul_rn(v.x, alpha));
}

// The top-hat filter applied to a spectrum value, rounded as two products
// (no contraction into the transform's first additions, so every pipeline
// filters with the same bits).
__device__ __forceinline__ float2 filter_mul(float2 z, float w) {
  return make_float2(__fmul_rn(z.x, w), __fmul_rn(z.y, w));
}

// Signed frequency index of position i on an N-point axis (:309-311).
__device__ __forceinline__ int kfreq(int i, int N) { return i > N / 2 ? i - N : i; }

}  // namespace sf21
