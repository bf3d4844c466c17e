// The plain GPU form of the HII filter bank: one radius per launch sequence,
// with the reference's structure (get_HIIbubbles.c:298-462) kept step by step
// -- filtered inverse transform, centre mask, and for R >= 2 dx the FP32 FFT
// convolution of the centre mask with the discrete sphere thresholded at 1/100
// of a count (:358-393); for R < 2 dx the ball painting (:427-458).  It is the
// baseline the batched form is measured against, and a second FP32 path with
// the reference's own dilation arithmetic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_kernels.h"
#include "softdouble.h"

namespace sf21 {

constexpr int EL_THREADS = 256;

// periodic index for any side N
__device__ __forceinline__ int pwrap(int x, int N) {
  x %= N;
  return x < 0 ? x + N : x;
}

static unsigned el_grid(long n) {
  long b = (n + EL_THREADS - 1) / EL_THREADS;
  return (unsigned)(b < 152 * 32 ? b : 152 * 32);
}

// Centre mask of the filtered packed box (:335-352, is_centre); flag = 1 if
// any.
__global__ void k_plain_centres(long n3, const float2* __restrict__ box, const float* __restrict__ alpha_ptr,
                                float zmul, float* __restrict__ mask, int* __restrict__ flag) {
  const float alpha = *alpha_ptr;
  int any = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const bool c = is_centre(box[i], alpha, zmul);
    mask[i] = c ? 1.0f : 0.0f;
    any |= c;
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Packed (sphere + i * centres) box for the convolution (:363-371): sphere =
// 1 where the minimum-image squared lattice distance n <= nmax.
__global__ void k_plain_pack_sphere(int N, int nmax, const float* __restrict__ mask,
                                    const int* __restrict__ flag, float2* __restrict__ out) {
  if (!*flag) return;
  const long n3 = (long)N * N * N;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const int a = (int)(i / ((long)N * N)), b = (int)((i / N) % N), c = (int)(i % N);
    const int da = a < N - a ? a : N - a, db = b < N - b ? b : N - b, dc = c < N - c ? c : N - c;
    const long n = (long)da * da + (long)db * db + (long)dc * dc;
    out[i] = make_float2(n <= nmax ? 1.0f : 0.0f, mask[i]);
  }
}

// P(k) = S(k) C(k) from Z = FFT(s + i c): S = (Z(k) + conj Z(-k))/2,
// C = (Z(k) - conj Z(-k))/(2i)   (the product of :379-381).
__global__ void k_plain_product(int N, const float2* __restrict__ Z, const int* __restrict__ flag,
                                float2* __restrict__ P) {
  if (!*flag) return;
  const long n3 = (long)N * N * N;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const int a = (int)(i / ((long)N * N)), b = (int)((i / N) % N), c = (int)(i % N);
    const long j = ((long)(a ? N - a : 0) * N + (b ? N - b : 0)) * N + (c ? N - c : 0);
    const float2 z = Z[i], w = Z[j];
    const float2 s = make_float2(0.5f * (z.x + w.x), 0.5f * (z.y - w.y));
    // (z - conj w) / (2i) = ((z.y + w.y) / 2, -(z.x - w.x) / 2)
    const float2 q = make_float2(0.5f * (z.y + w.y), -0.5f * (z.x - w.x));
    P[i] = make_float2(s.x * q.x - s.y * q.y, s.x * q.y + s.y * q.x);
  }
}

// Threshold of the convolution (:390-393): count = conv / N^3 > 1/100.
__global__ void k_plain_threshold(long n3, const float2* __restrict__ conv, const int* __restrict__ flag,
                                  float* __restrict__ bubblef) {
  if (!*flag) return;
  const float inv = 1.0f / (float)n3;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x)
    if (conv[i].x * inv > 0.01f) bubblef[i] = 1.0f;
}

// Small-R painting (:433-458) as a gather: voxel y is painted if a centre
// lies at an offset with squared length <= nmax (offsets within +-(nc+1)).
__global__ void k_plain_paint(int N, int nc, int nmax, const float* __restrict__ mask,
                              float* __restrict__ bubblef) {
  const long n3 = (long)N * N * N;
  const int w = nc + 1;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const int a = (int)(i / ((long)N * N)), b = (int)((i / N) % N), c = (int)(i % N);
    bool hit = false;
    for (int da = -w; da <= w && !hit; ++da)
      for (int db = -w; db <= w && !hit; ++db)
        for (int dc = -w; dc <= w && !hit; ++dc) {
          if (da * da + db * db + dc * dc > nmax) continue;
          const long j = ((long)pwrap(a - da, N) * N + pwrap(b - db, N)) * N + pwrap(c - dc, N);
          hit = mask[j] != 0.0f;
        }
    if (hit) bubblef[i] = 1.0f;
  }
}

// Cap (:469-471) in exact double arithmetic.
__global__ void k_plain_cap(long n3, const float* __restrict__ fres, float* __restrict__ bubblef) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const sd_t om = sd_sub(0x3FF0000000000000ULL, sd_from_float(fres[i]));
    if (sd_gt(sd_from_float(bubblef[i]), om)) bubblef[i] = sd_to_float(om);
  }
}

cudaError_t launch_plain_centres(long n3, const float2* box, const float* alpha, float zmul, float* mask, int* flag,
                                 cudaStream_t st) {
  k_plain_centres<<<el_grid(n3), EL_THREADS, 0, st>>>(n3, box, alpha, zmul, mask, flag);
  return cudaGetLastError();
}
cudaError_t launch_plain_pack_sphere(int N, int nmax, const float* mask, const int* flag, float2* out,
                                     cudaStream_t st) {
  k_plain_pack_sphere<<<el_grid((long)N * N * N), EL_THREADS, 0, st>>>(N, nmax, mask, flag, out);
  return cudaGetLastError();
}
cudaError_t launch_plain_product(int N, const float2* Z, const int* flag, float2* P, cudaStream_t st) {
  k_plain_product<<<el_grid((long)N * N * N), EL_THREADS, 0, st>>>(N, Z, flag, P);
  return cudaGetLastError();
}
cudaError_t launch_plain_threshold(long n3, const float2* conv, const int* flag, float* bubblef, cudaStream_t st) {
  k_plain_threshold<<<el_grid(n3), EL_THREADS, 0, st>>>(n3, conv, flag, bubblef);
  return cudaGetLastError();
}
cudaError_t launch_plain_paint(int N, int nc, int nmax, const float* mask, float* bubblef, cudaStream_t st) {
  k_plain_paint<<<el_grid((long)N * N * N), EL_THREADS, 0, st>>>(N, nc, nmax, mask, bubblef);
  return cudaGetLastError();
}
cudaError_t launch_plain_cap(long n3, const float* fres, float* bubblef, cudaStream_t st) {
  k_plain_cap<<<el_grid(n3), EL_THREADS, 0, st>>>(n3, fres, bubblef);
  return cudaGetLastError();
}

}  // namespace sf21
