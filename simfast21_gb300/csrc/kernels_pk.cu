// Power spectrum of a cubic box on the GPU (tools/power3d_f.c:124-194):
// window, forward transform (the filter bank's own FFT passes), and the
// spherical binning of |F(k)|^2 over the r2c half-spectrum.
//
//   k_pk_pack: (float)(value * w(i) w(j) w(p)) as the real part of a complex
//     box (imaginary part 0), the window given per axis;
//   k_pk_bin: one CTA per PK_ROWS rows (i, j), threads over p = 0..N/2:
//     bin = round(|k| / dk) = round(sqrt(i'^2 + j'^2 + p^2)) in integers
//     (i', j' the signed indices; for a cube every axis has the same dk),
//     power = re^2 + im^2 in float as the tool computes it; per-CTA sums in
//     shared memory, written out per CTA and added up in double on the host,
//     counts added exactly with integer atomics.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

constexpr int PK_THREADS = 256;
constexpr int PK_ROWS = 32;

int pk_nbins(int N) {
  const long h = N / 2;
  long m = 0;
  const long n = 3 * h * h;
  while ((m + 1) * (m + 1) <= n) ++m;
  return (int)((n - m * m > m) ? m + 1 : m) + 1;  // round(sqrt(3 (N/2)^2)) + 1, :83
}

int pk_bin_grid(int N) { return (int)(((long)N * N + PK_ROWS - 1) / PK_ROWS); }

__global__ void k_pk_pack(long n3, int N, const float* __restrict__ box, const float* __restrict__ wax,
                          float2* __restrict__ out) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n3; t += (long)gridDim.x * blockDim.x) {
    const int p = (int)(t % N), j = (int)((t / N) % N), i = (int)(t / ((long)N * N));
    const float w = __fmul_rn(__fmul_rn(wax[i], wax[j]), wax[p]);
    out[t] = make_float2(__fmul_rn(box[t], w), 0.0f);
  }
}

__device__ __forceinline__ int round_sqrt(int n) {
  int m = (int)sqrtf((float)n);
  while (m * m > n) --m;
  while ((m + 1) * (m + 1) <= n) ++m;
  return (n - m * m > m) ? m + 1 : m;  // sqrt(n) >= m + 1/2  <=>  n > m^2 + m
}

__global__ void __launch_bounds__(PK_THREADS)
k_pk_bin(int N, const float2* __restrict__ spec, int nk, float* __restrict__ partials,
         unsigned long long* __restrict__ counts) {
  extern __shared__ float pk_smem[];
  float* sums = pk_smem;
  int* cnt = reinterpret_cast<int*>(pk_smem + nk);
  for (int b = threadIdx.x; b < nk; b += blockDim.x) {
    sums[b] = 0.0f;
    cnt[b] = 0;
  }
  __syncthreads();
  const int half = N / 2 + 1;
  const long row0 = (long)blockIdx.x * PK_ROWS;
  for (int t = threadIdx.x; t < PK_ROWS * half; t += blockDim.x) {
    const long row = row0 + t / half;
    if (row >= (long)N * N) break;
    const int p = t % half;
    const int i = (int)(row / N), j = (int)(row % N);
    const int si = kfreq(i, N), sj = kfreq(j, N);
    const int b = round_sqrt(si * si + sj * sj + p * p);
    const float2 z = spec[row * N + p];
    const float pw = __fadd_rn(__fmul_rn(z.x, z.x), __fmul_rn(z.y, z.y));
    atomicAdd(&sums[b], pw);
    atomicAdd(&cnt[b], 1);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nk; b += blockDim.x) {
    partials[(long)blockIdx.x * nk + b] = sums[b];
    if (cnt[b]) atomicAdd(&counts[b], (unsigned long long)cnt[b]);
  }
}

cudaError_t launch_pk_pack(int N, const float* box, const float* wax, float2* out, cudaStream_t st) {
  const long n3 = (long)N * N * N;
  long blocks = (n3 + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_pk_pack<<<(unsigned)blocks, 256, 0, st>>>(n3, N, box, wax, out);
  return cudaGetLastError();
}

cudaError_t launch_pk_bin(int N, const float2* spec, int nk, float* partials, unsigned long long* counts,
                          cudaStream_t st) {
  const size_t smem = (size_t)nk * (sizeof(float) + sizeof(int));
  k_pk_bin<<<pk_bin_grid(N), PK_THREADS, smem, st>>>(N, spec, nk, partials, counts);
  return cudaGetLastError();
}

}  // namespace sf21
