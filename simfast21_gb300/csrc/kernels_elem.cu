// Element-wise kernels of the HII stage: the prologue
// (get_HIIbubbles.c:216-225, 272-274), the norm balance of the packed
// transform and the single-cell fill check hook (:281-288).  All per-voxel
// double arithmetic of the reference is reproduced bit for bit with the
// integer soft-double routines.  The dilation and the per-set finish are in
// kernels_dt.cu.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_kernels.h"
#include "softdouble.h"

namespace sf21 {

#define SD_ONE (0x3FF0000000000000ULL)

// Source chain before zeta, left to right as the reference multiplies.
__device__ __forceinline__ sd_t src_chain(float s, const PrologueArgs& pa) {
  sd_t t = sd_from_float(s);
  for (int m = 0; m < pa.n_src_mul; ++m) t = sd_mul(t, pa.src_mul[m]);
  return t;
}

constexpr int PRO_THREADS = 256;

__global__ void __launch_bounds__(PRO_THREADS)
k_prologue(long n3, const float* __restrict__ delta, const float* __restrict__ src,
           const PrologueArgs pa, float* __restrict__ rec0, float* __restrict__ fres,
           float2* __restrict__ packed, float* __restrict__ partials) {
  float sd2 = 0.f, sh2 = 0.f;
  int nz = 0;  // some ionisation rate is not exactly zero
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const float d = delta[i];
    const sd_t one_d = sd_add(SD_ONE, sd_from_float(d));  // 1. + density_map[i]
    // Each quantity takes its fast path (prologue_fast.h), which returns the
    // exact chain's float for all but about one voxel in 2^21; those voxels
    // evaluate the exact chain.
    // fresid = XHI((float)((1+d) * 1.881e-7 * pow(1+z,3) * G_H(z)))      (:220-221)
    float fr;
    if (!prod_fast(one_d, pa.pf_resid, &fr))
      fr = sd_to_float(sd_mul(sd_mul(sd_mul(one_d, pa.c_resid), pa.one_plus_z_cubed), pa.g_h));
    const float fx = xhi_float(fr);
    // density_map = (float)Rrec((float)(1 + d), z)                          (:222)
    const float od = sd_to_float(one_d);
    float rr;
    if (!rrec_fast(od, pa.rf, &rr))
      rr = sd_to_float(rrec_exact(od, pa.r2c, pa.r3, pa.rec1, pa.dvv, pa.v_normc));
    // source before zeta                                                   (:272-274)
    const float s = src[i];
    float h1;
    if (!prod_fast(sd_from_float(s), pa.pf_src, &h1)) h1 = sd_to_float(src_chain(s, pa));
    rec0[i] = rr;
    fres[i] = fx;
    packed[i] = make_float2(rr, h1);
    sd2 += rr * rr;
    sh2 += h1 * h1;
    nz |= (h1 != 0.0f);
  }
  nz = __syncthreads_or(nz);
  // block reduction of the two sums of squares (only their ratio is used)
  __shared__ float red[2][PRO_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    sd2 += __shfl_xor_sync(0xffffffffu, sd2, o);
    sh2 += __shfl_xor_sync(0xffffffffu, sh2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = sd2;
    red[1][threadIdx.x >> 5] = sh2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int w = 0; w < PRO_THREADS / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    // a block with a nonzero rate reports a nonzero sum even when every
    // square underflows, so that an all-zero box is told apart exactly
    if (nz && b == 0.f) b = __int_as_float(1);
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

int prologue_blocks(long n3) {
  long b = (n3 + PRO_THREADS - 1) / PRO_THREADS;
  return (int)(b < 152 * 16 ? b : 152 * 16);
}

cudaError_t launch_prologue(long n3, const float* delta, const float* src, const PrologueArgs& pa,
                            float* rec0, float* fres, float2* packed, float* partials, int nblocks,
                            cudaStream_t st) {
  k_prologue<<<nblocks, PRO_THREADS, 0, st>>>(n3, delta, src, pa, rec0, fres, packed, partials);
  return cudaGetLastError();
}

// alpha = 2^round(log2(|rec| / |ion|)), so that the two halves of the packed
// transform have comparable norms.  An ionisation box that is zero in every
// cell gets alpha = -1: the reference's filtered ionisation field is then
// exactly zero and no cell is a centre (its test wants ion_R > 0,
// get_HIIbubbles.c:339-348), while the packed transform's imaginary half
// holds rounding cross-talk from the recombination half; is_centre reads
// alpha <= 0 as "no centre", and the other users take |alpha|.
__global__ void k_alpha(const float* __restrict__ partials, int nblocks, float* __restrict__ alpha) {
  __shared__ float sa[256], sb[256];
  float a = 0.f, b = 0.f;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
    a += partials[2 * i];
    b += partials[2 * i + 1];
  }
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    float r = 1.0f;
    if (sb[0] == 0.f) {
      r = -1.0f;
    } else if (sa[0] > 0.f && sb[0] > 0.f && isfinite(sa[0]) && isfinite(sb[0])) {
      float e = rintf(0.5f * log2f(sa[0] / sb[0]));
      e = fminf(fmaxf(e, -60.f), 60.f);
      r = exp2f(e);
    }
    *alpha = r;
  }
}

cudaError_t launch_alpha(const float* partials, int nblocks, float* alpha, cudaStream_t st) {
  k_alpha<<<1, 256, 0, st>>>(partials, nblocks, alpha);
  return cudaGetLastError();
}

// Single-cell fill alone (check hook): :281-288 without dilation and cap.
__global__ void k_fill0(long n3, sd_t zeta, const float* __restrict__ src, const float* __restrict__ rec0,
                        const PrologueArgs pa, float* __restrict__ fill) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const float h = sd_to_float(sd_mul(src_chain(src[i], pa), zeta));
    const float d = rec0[i];
    float f;
    if (h > 0.0f)
      f = (d > 0.0f) ? ((h >= d) ? 1.0f : __fdiv_rn(h, d)) : 1.0f;
    else
      f = 0.0f;
    fill[i] = f;
  }
}

cudaError_t launch_fill0(long n3, uint64_t zeta, const float* src, const float* rec0,
                         const PrologueArgs& pa, float* fill, cudaStream_t st) {
  k_fill0<<<prologue_blocks(n3), PRO_THREADS, 0, st>>>(n3, zeta, src, rec0, pa, fill);
  return cudaGetLastError();
}

}  // namespace sf21
