// 21-cm brightness temperature on the GPU (t21.c:114-255): the line-of-sight
// velocity gradient of the density box through the filter bank's FFT passes
// and the per-voxel brightness temperature.
//
//   k_t21_pack:    density -> complex box (imaginary part 0);
//   k_t21_kfilter: spectrum times k_axis^2 / k^2 (0 at k = 0), full complex
//                  spectrum in natural order, signed indices (the factor is
//                  even in k, so the inverse stays real, as the reference's
//                  c2r of the half-spectrum);
//   k_t21_finish:  dv = scale * Re(inverse), clamped to [-0.5, 1]; spin
//                  factor (1, or x/(1+x) (1 - Tcmb/TK) with x = xc + xalpha);
//                  T_b = pref (1 + delta) t / (1 + dv) (1 - xHII); per-block
//                  float sums of T_b and of Tcmb/(1 - t), added up in double on
//                  the host.
// Single precision throughout (the reference computes in double; the
// differences are at the float rounding of the output).
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

constexpr int T21_THREADS = 256;

int t21_blocks(long n3) {
  long b = (n3 + T21_THREADS - 1) / T21_THREADS;
  return (int)(b < 152 * 16 ? b : 152 * 16);
}

__global__ void k_t21_pack(long n3, const float* __restrict__ delta, float2* __restrict__ out) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n3; t += (long)gridDim.x * blockDim.x)
    out[t] = make_float2(delta[t], 0.0f);
}

__global__ void k_t21_kfilter(int N, int axis, float2* __restrict__ spec) {
  const long n3 = (long)N * N * N;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n3; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % N), j = (int)((t / N) % N), i = (int)(t / ((long)N * N));
    const int si = kfreq(i, N), sj = kfreq(j, N), sp = kfreq(p, N);
    const int k2 = si * si + sj * sj + sp * sp;
    const int a = axis == 1 ? si : (axis == 2 ? sj : sp);
    const float g = k2 ? __fdiv_rn((float)(a * a), (float)k2) : 0.0f;
    const float2 z = spec[t];
    spec[t] = make_float2(z.x * g, z.y * g);
  }
}

__global__ void __launch_bounds__(T21_THREADS)
k_t21_finish(long n3, const float2* __restrict__ inv, const float* __restrict__ delta,
             const float* __restrict__ xhii, const float* __restrict__ xc, const float* __restrict__ xalpha,
             const float* __restrict__ tempx, T21Args ta, float* __restrict__ tb, float* __restrict__ partials) {
  float s_tb = 0.f, s_ts = 0.f;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n3; t += (long)gridDim.x * blockDim.x) {
    float dv = ta.scale * inv[t].x;
    if (dv > 1.0f) dv = 1.0f;
    else if (dv < -0.5f) dv = -0.5f;
    float s = 1.0f;
    if (xc) {
      const float x = xalpha[t] + xc[t];
      s = x / (1.0f + x);
      s = s * (1.0f - ta.tcmb / tempx[t]);
      s_ts += ta.tcmb / (1.0f - s);
    }
    const float v = ta.pref * (1.0f + delta[t]) * s / (1.0f + dv) * (1.0f - xhii[t]);
    tb[t] = v;
    s_tb += v;
  }
  __shared__ float red[2][T21_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s_tb += __shfl_xor_sync(0xffffffffu, s_tb, o);
    s_ts += __shfl_xor_sync(0xffffffffu, s_ts, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s_tb;
    red[1][threadIdx.x >> 5] = s_ts;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int w = 0; w < T21_THREADS / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

cudaError_t launch_t21_pack(long n3, const float* delta, float2* out, cudaStream_t st) {
  k_t21_pack<<<t21_blocks(n3), T21_THREADS, 0, st>>>(n3, delta, out);
  return cudaGetLastError();
}

cudaError_t launch_t21_kfilter(int N, int axis, float2* spec, cudaStream_t st) {
  k_t21_kfilter<<<t21_blocks((long)N * N * N), T21_THREADS, 0, st>>>(N, axis, spec);
  return cudaGetLastError();
}

cudaError_t launch_t21_finish(long n3, const float2* inv, const float* delta, const float* xhii, const float* xc,
                              const float* xalpha, const float* tempx, const T21Args& ta, float* tb,
                              float* partials, cudaStream_t st) {
  k_t21_finish<<<t21_blocks(n3), T21_THREADS, 0, st>>>(n3, inv, delta, xhii, xc, xalpha, tempx, ta, tb, partials);
  return cudaGetLastError();
}

}  // namespace sf21
