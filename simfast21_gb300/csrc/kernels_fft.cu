// 3D FFT passes of the HII filter bank (sm_103a).
//
// Layout: an N^3 complex64 box, index (a, b, c) = a N^2 + b N + c, c fastest.
// The packed field z = rec + i * alpha * ion carries the recombination-rate
// box (get_HIIbubbles.c:222) and the ionisation-rate box (:273) together: the
// top-hat filter is real and even, so one complex transform of z replaces the
// reference's two real transforms (pr2c1/pr2c2 at :290-291 and pc2r1/pc2r2
// at :324-325, :424-425) and its real and imaginary parts are the two
// filtered fields.  alpha is a power of two that balances the two norms so
// neither field drowns in the other's rounding; it cancels exactly in the
// centre test.
//
// Passes:
//   c-axis (contiguous rows): coalesced row loads straight into registers;
//     the inverse variant reads the spectrum once and emits K filtered,
//     c-transformed work boxes (one per radius of the batch);
//   b- and a-axis (strided): a tile of N rows x CW contiguous columns, each
//     column a line of the FFT;
//   the a-axis inverse pass ends in the centre test (:335-352, :437-438) and
//     the first-hit radius update, so filtered fields never go back to HBM.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

// ---------------------------------------------------------------------------
// Forward c-axis pass of the packed prologue output: z = (rec0, ion * alpha).
template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS)
k_fwd_rows(const float2* __restrict__ in, float2* __restrict__ out,
           const float* __restrict__ alpha_ptr, const float2* __restrict__ gtw) {
  using G = RowGeom<N>;
  using L = LineGeom<N>;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[G::ROWS * L::LS];
  load_twiddles<N>(stw, gtw);
  const int row_in_cta = threadIdx.x / G::T;
  const int j = threadIdx.x % G::T;
  const long row = (long)blockIdx.x * G::ROWS + row_in_cta;
  const float alpha = alpha_ptr ? fabsf(*alpha_ptr) : 1.0f;
  float2 v[8];
  const float2* src = in + row * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    float2 x = src[j + r * (N / 8)];
    x.y *= alpha;
    v[r] = x;
  }
  __syncthreads();
  fft_line<N, false>(v, sbuf + row_in_cta * L::LS, stw, j);
  float2* dst = out + row * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) dst[j + r * (N / 8)] = v[r];
}

// ---------------------------------------------------------------------------
// Inverse c-axis pass with the k-space top-hat filter of K radii
// (get_HIIbubbles.c:305-322): the spectrum row is read once, then for each
// radius multiplied by W(dk R |k|) and transformed into its work box.
template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS)
k_inv_rows_filter(const float2* __restrict__ spec, Batch bt, const float2* __restrict__ gtw) {
  using G = RowGeom<N>;
  using L = LineGeom<N>;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[G::ROWS * L::LS];
  load_twiddles<N>(stw, gtw);
  const int row_in_cta = threadIdx.x / G::T;
  const int j = threadIdx.x % G::T;
  const long row = (long)blockIdx.x * G::ROWS + row_in_cta;
  const int a = (int)(row / N), b = (int)(row % N);
  const int ka = kfreq(a, N), kb = kfreq(b, N);
  const int kab = ka * ka + kb * kb;
  float2 z[8];
  float kmag[8];
  const float2* src = spec + row * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int c = j + r * (N / 8);
    z[r] = src[c];
    const int kc = kfreq(c, N);
    kmag[r] = sqrtf((float)(kab + kc * kc));
  }
  __syncthreads();
  for (int k = 0; k < bt.K; ++k) {
    const float dkR = bt.r[k].dkR;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float w = w_tophat(dkR * kmag[r]);
      v[r] = filter_mul(z[r], w);
    }
    fft_line<N, true>(v, sbuf + row_in_cta * L::LS, stw, j);
    float2* dst = bt.r[k].work + row * N;
#pragma unroll
    for (int r = 0; r < 8; ++r) dst[j + r * (N / 8)] = v[r];
  }
}

// Unfiltered inverse c-axis pass in place (plain form and tests).
template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS)
k_inv_rows_plain(float2* __restrict__ box, const float2* __restrict__ gtw) {
  using G = RowGeom<N>;
  using L = LineGeom<N>;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[G::ROWS * L::LS];
  load_twiddles<N>(stw, gtw);
  const int row_in_cta = threadIdx.x / G::T;
  const int j = threadIdx.x % G::T;
  const long row = (long)blockIdx.x * G::ROWS + row_in_cta;
  float2 v[8];
  float2* p = box + row * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = p[j + r * (N / 8)];
  __syncthreads();
  fft_line<N, true>(v, sbuf + row_in_cta * L::LS, stw, j);
#pragma unroll
  for (int r = 0; r < 8; ++r) p[j + r * (N / 8)] = v[r];
}

// ---------------------------------------------------------------------------
// Strided-axis pass in place: AXIS 1 = b (stride N), AXIS 0 = a (stride N^2).
// blockIdx.x enumerates (outer index, column block); blockIdx.y selects the
// box (work box of radius y of the batch, or the single box `box0`).
template <int N, bool INV>
__global__ void __launch_bounds__(ColGeom<N>::THREADS)
k_cols(float2* box0, Batch bt, int axis, const float2* __restrict__ gtw) {
  using C = ColGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  load_twiddles<N>(stw, gtw);
  float2* box = box0 ? box0 : bt.r[blockIdx.y].work;
  const int nblk = N / C::CW;
  const int outer = blockIdx.x / nblk;
  const int c0 = (blockIdx.x % nblk) * C::CW;
  const long stride = axis == 1 ? (long)N : (long)N * N;
  const long base = (axis == 1 ? (long)outer * N * N : (long)outer * N) + c0;
  const int col = threadIdx.x % C::CW;
  const int j = threadIdx.x / C::CW;
  float2 v[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = box[base + (long)(j + r * (N / 8)) * stride + col];
  __syncthreads();
  fft_line<N, INV>(v, sbuf + col * L::LS, stw, j);
#pragma unroll
  for (int r = 0; r < 8; ++r) box[base + (long)(j + r * (N / 8)) * stride + col] = v[r];
}

// ---------------------------------------------------------------------------
// Last inverse pass (a axis) of a batch, fused with the centre test and the
// first-hit radius update.  Each CTA runs all K radii of the batch on the
// same tile, keeps the smallest radius index at which each voxel is a centre
// and updates rc (uint8 per voxel of the set) once (centre test: is_centre).
template <int N>
__global__ void __launch_bounds__(ColGeom<N>::THREADS)
k_cols_a_test(Batch bt, uint8_t* __restrict__ rc, const float* __restrict__ alpha_ptr,
              const float2* __restrict__ gtw) {
  using C = ColGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  load_twiddles<N>(stw, gtw);
  const float alpha = *alpha_ptr;
  const int nblk = N / C::CW;
  const int b = blockIdx.x / nblk;
  const int c0 = (blockIdx.x % nblk) * C::CW;
  const long stride = (long)N * N;
  const long base = (long)b * N + c0;
  const int col = threadIdx.x % C::CW;
  const int j = threadIdx.x / C::CW;
  int hit[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) hit[r] = RC_NONE;
  for (int k = 0; k < bt.K; ++k) {
    const float2* box = bt.r[k].work;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = box[base + (long)(j + r * (N / 8)) * stride + col];
    __syncthreads();
    fft_line<N, true>(v, sbuf + col * L::LS, stw, j);
    const int ridx = bt.r[k].ridx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (is_centre(v[r], alpha, bt.zmul) && ridx < hit[r]) hit[r] = ridx;
    }
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    if (hit[r] != RC_NONE) {
      const long idx = base + (long)(j + r * (N / 8)) * stride + col;
      const uint8_t old = rc[idx];
      if (hit[r] < old) rc[idx] = (uint8_t)hit[r];
    }
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers (dispatch on N), one per kernel so that the caller can
// put timing events between them.
template <int N>
struct Launch {
  static constexpr size_t smem_cols() { return (N + ColGeom<N>::CW * LineGeom<N>::LS) * sizeof(float2); }
  static unsigned grid_rows() { return (unsigned)((long)N * N / RowGeom<N>::ROWS); }
  static unsigned grid_cols() { return (unsigned)((long)N * (N / ColGeom<N>::CW)); }
  static cudaError_t fwd_rows(const float2* in, float2* out, const float* alpha, const float2* tw, cudaStream_t st) {
    k_fwd_rows<N><<<grid_rows(), RowGeom<N>::THREADS, 0, st>>>(in, out, alpha, tw);
    return cudaGetLastError();
  }
  static cudaError_t inv_rows_plain(float2* box, const float2* tw, cudaStream_t st) {
    k_inv_rows_plain<N><<<grid_rows(), RowGeom<N>::THREADS, 0, st>>>(box, tw);
    return cudaGetLastError();
  }
  static cudaError_t inv_rows_filter(const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st) {
    k_inv_rows_filter<N><<<grid_rows(), RowGeom<N>::THREADS, 0, st>>>(spec, bt, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols(float2* box, const Batch& bt, int nbox, int axis, bool inv, const float2* tw,
                          cudaStream_t st) {
    if (inv)
      k_cols<N, true><<<dim3(grid_cols(), nbox), ColGeom<N>::THREADS, smem_cols(), st>>>(box, bt, axis, tw);
    else
      k_cols<N, false><<<dim3(grid_cols(), nbox), ColGeom<N>::THREADS, smem_cols(), st>>>(box, bt, axis, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols_a_test(const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                                 cudaStream_t st) {
    k_cols_a_test<N><<<grid_cols(), ColGeom<N>::THREADS, smem_cols(), st>>>(bt, rc, alpha, tw);
    return cudaGetLastError();
  }
  static cudaError_t setup() {
    const int smem = (int)smem_cols();
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_cols<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))) return e;
    if ((e = cudaFuncSetAttribute(k_cols<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))) return e;
    if ((e = cudaFuncSetAttribute(k_cols_a_test<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))) return e;
    return cudaSuccess;
  }
};

#define SF21_DISPATCH_N(N, CALL)                         \
  switch (N) {                                           \
    case 16: { using LL = Launch<16>; return CALL; }     \
    case 32: { using LL = Launch<32>; return CALL; }     \
    case 64: { using LL = Launch<64>; return CALL; }     \
    case 128: { using LL = Launch<128>; return CALL; }   \
    case 256: { using LL = Launch<256>; return CALL; }   \
    case 512: { using LL = Launch<512>; return CALL; }   \
    case 1024: { using LL = Launch<1024>; return CALL; } \
    default: return cudaErrorInvalidValue;               \
  }

cudaError_t fft_setup(int N) { SF21_DISPATCH_N(N, LL::setup()); }
cudaError_t launch_fwd_rows(int N, const float2* in, float2* out, const float* alpha, const float2* tw,
                            cudaStream_t st) {
  SF21_DISPATCH_N(N, LL::fwd_rows(in, out, alpha, tw, st));
}
cudaError_t launch_inv_rows_plain(int N, float2* box, const float2* tw, cudaStream_t st) {
  SF21_DISPATCH_N(N, LL::inv_rows_plain(box, tw, st));
}
cudaError_t launch_inv_rows_filter(int N, const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st) {
  SF21_DISPATCH_N(N, LL::inv_rows_filter(spec, bt, tw, st));
}
cudaError_t launch_cols(int N, float2* box, const Batch& bt, int nbox, int axis, bool inverse, const float2* tw,
                        cudaStream_t st) {
  SF21_DISPATCH_N(N, LL::cols(box, bt, nbox, axis, inverse, tw, st));
}
cudaError_t launch_cols_a_test(int N, const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                               cudaStream_t st) {
  SF21_DISPATCH_N(N, LL::cols_a_test(bt, rc, alpha, tw, st));
}

}  // namespace sf21
