// Inverse transform of a batch in the column-block-major work layout.
//
// The work boxes of a batch are intermediates, so their layout is free.  In
// the natural layout (a N^2 + b N + c) the a-axis pass reads rows of CW
// contiguous columns N^2 elements apart: one tile touches N different 2 MB
// pages of an N^3 box, which thrashes the GPU's address-translation caches.
// Here the boxes are stored column-block major,
//     index(a, b, c) = ((c / CW) N + a) N + b) CW + c mod CW,
// i.e. one slab of N^2 x CW values per column block.  Then
//   * the c-axis pass (filter + inverse c transform) writes each row as N/CW
//     runs of CW contiguous values;
//   * a b-axis tile (fixed a, one column block) is one contiguous N CW run;
//   * an a-axis tile (fixed b, one column block) reads N runs of CW values
//     N CW apart, inside one N^2 CW slab (32 MB at N = 512).
// The centre test and the first-hit update write rc in the natural layout.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

template <int N>
struct CbGeom {
  static constexpr int CW = (N <= 512) ? 16 : 8;  // columns per block (CW * 8 bytes per run)
  static constexpr int NBLK = N / CW;
  static constexpr int RT = N / 8;                // threads per row (c-axis pass)
  static constexpr int ROWS = (256 / RT) > 0 ? (256 / RT) : 1;
  static constexpr int RTHREADS = RT * ROWS;
};

template <int N>
__device__ __forceinline__ long cb_index(int a, int b, int c) {
  using G = CbGeom<N>;
  return (((long)(c / G::CW) * N + a) * N + b) * G::CW + (c % G::CW);
}

// c-axis inverse pass with the top-hat filter of the K radii of the batch
// (get_HIIbubbles.c:305-322): spectrum row (a, b) read once, K filtered
// transformed rows written column-block major.
template <int N>
__global__ void __launch_bounds__(CbGeom<N>::RTHREADS)
k_rows_filter_cb(const float2* __restrict__ spec, Batch bt, const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using L = LineGeom<N>;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[G::ROWS * L::LS];
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int row_in_cta = threadIdx.x / G::RT;
  const int j = threadIdx.x % G::RT;
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
      v[r] = make_float2(z[r].x * w, z[r].y * w);
    }
    fft_line<N, true>(v, sbuf + row_in_cta * L::LS, stw, j);
    if constexpr ((N / 8) % G::CW == 0) {
      // c = j + r N/8: column block j/CW + r (N/8)/CW, offset j mod CW
      float2* dst = bt.r[k].work + cb_index<N>(a, b, j);
      constexpr long RSTRIDE = (long)(N / 8 / G::CW) * N * N * G::CW;
#pragma unroll
      for (int r = 0; r < 8; ++r) dst[r * RSTRIDE] = v[r];
    } else {
      float2* dst = bt.r[k].work;
#pragma unroll
      for (int r = 0; r < 8; ++r) dst[cb_index<N>(a, b, j + r * (N / 8))] = v[r];
    }
  }
}

// b-axis inverse pass in place: tile (a, column block) is one contiguous run
// of N CW values per radius.  A CTA takes KW of the CW columns and walks the K
// radii, issuing the loads of radius k + 1 before the transform of radius k.
// blockIdx.x = (cb N + a) (CW / KW) + column half.
// (A CTA takes the whole column block: with 16 columns a warp covers 16
// lines x 2 threads, whose shared-memory exchanges of the line FFT are free of
// bank conflicts; 8-column CTAs conflicted and stalled on the MIO pipe.)
template <int N>
struct KGeom {
  static constexpr int KW = CbGeom<N>::CW;  // columns per CTA
  static constexpr int SPLIT = CbGeom<N>::CW / KW;
  static constexpr int THREADS = KW * (N / 8);
  static constexpr size_t SMEM = (size_t)(N + KW * LineGeom<N>::LS) * sizeof(float2);
};

template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, (KGeom<N>::THREADS <= 512 ? 2 : 1))
k_cols_b_cb(Batch bt, const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using X = KGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int tile = blockIdx.x / X::SPLIT;
  const int half = blockIdx.x % X::SPLIT;
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const long off = (long)tile * N * G::CW + half * X::KW + col;  // element (b = 0) of this column
  float2 v[8], nx[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = bt.r[0].work[off + (j + r * (N / 8)) * G::CW];
  for (int k = 0; k < bt.K; ++k) {
    if (k + 1 < bt.K) {
      const float2* nbox = bt.r[k + 1].work + off;
#pragma unroll
      for (int r = 0; r < 8; ++r) nx[r] = nbox[(j + r * (N / 8)) * G::CW];
    }
    __syncthreads();
    fft_line<N, true>(v, sbuf + col * L::LS, stw, j);
    float2* box = bt.r[k].work + off;
#pragma unroll
    for (int r = 0; r < 8; ++r) box[(j + r * (N / 8)) * G::CW] = v[r];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = nx[r];
  }
}

// a-axis inverse pass of the K radii + centre test + first-hit update
// (get_HIIbubbles.c:335-352; for floats h, d > 0, (double)h/d >= 1 <=> h >= d).
// A CTA takes KW of the CW columns of one column block (fixed b) and walks
// the K radii; the loads of radius k + 1 are issued before the transform of
// radius k, so every warp keeps a tile in flight while it computes.
// blockIdx.x = (cb N + b) (CW / KW) + column half.
template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, (KGeom<N>::THREADS <= 512 ? 2 : 1))
k_cols_a_test_cb(Batch bt, uint8_t* __restrict__ rc, const float* __restrict__ alpha_ptr,
                 const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using X = KGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const float alpha = *alpha_ptr;
  const int tile = blockIdx.x / X::SPLIT;
  const int half = blockIdx.x % X::SPLIT;
  const int cb = tile / N;
  const int b = tile % N;
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const int cc = half * X::KW + col;                       // column within the block
  const long base = ((long)cb * N * N + b) * G::CW + cc;    // element (a = 0, b, cb CW + cc)
  const long astride = (long)N * G::CW;
  uint32_t hit_lo = 0xFFFFFFFFu, hit_hi = 0xFFFFFFFFu;      // 8 first-hit bytes
  float2 v[8], nx[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = bt.r[0].work[base + (long)(j + r * (N / 8)) * astride];
  for (int k = 0; k < bt.K; ++k) {
    if (k + 1 < bt.K) {
      const float2* nbox = bt.r[k + 1].work + base;
#pragma unroll
      for (int r = 0; r < 8; ++r) nx[r] = nbox[(long)(j + r * (N / 8)) * astride];
    }
    __syncthreads();
    fft_line<N, true>(v, sbuf + col * L::LS, stw, j);
    const uint32_t ridx = (uint32_t)bt.r[k].ridx;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float rec = v[r].x * alpha;  // alpha * rec_R (exact: power of two)
      const float ion = v[r].y * bt.zmul;
      const bool centre = (v[r].y > 0.0f) && (!(rec > 0.0f) || ion >= rec);
      uint32_t& h = r < 4 ? hit_lo : hit_hi;
      const int sh = 8 * (r & 3);
      if (centre && ridx < ((h >> sh) & 0xFFu)) h = (h & ~(0xFFu << sh)) | (ridx << sh);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = nx[r];
  }
  const int c = cb * G::CW + cc;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const uint32_t h = ((r < 4 ? hit_lo : hit_hi) >> (8 * (r & 3))) & 0xFFu;
    if (h != RC_NONE) {
      const long idx = ((long)(j + r * (N / 8)) * N + b) * N + c;
      const uint8_t old = rc[idx];
      if (h < old) rc[idx] = (uint8_t)h;
    }
  }
}

template <int N>
struct CbLaunch {
  using G = CbGeom<N>;
  static cudaError_t setup() {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_cols_b_cb<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KGeom<N>::SMEM)))
      return e;
    return cudaFuncSetAttribute(k_cols_a_test_cb<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)KGeom<N>::SMEM);
  }
  static cudaError_t rows(const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st) {
    k_rows_filter_cb<N><<<(unsigned)((long)N * N / G::ROWS), G::RTHREADS, 0, st>>>(spec, bt, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols_b(const Batch& bt, const float2* tw, cudaStream_t st) {
    using X = KGeom<N>;
    k_cols_b_cb<N><<<(unsigned)((long)N * G::NBLK * X::SPLIT), X::THREADS, X::SMEM, st>>>(bt, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols_a_test(const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                                 cudaStream_t st) {
    using X = KGeom<N>;
    k_cols_a_test_cb<N><<<(unsigned)((long)N * G::NBLK * X::SPLIT), X::THREADS, X::SMEM, st>>>(bt, rc, alpha, tw);
    return cudaGetLastError();
  }
};

#define SF21_CB_DISPATCH(N, CALL)                          \
  switch (N) {                                             \
    case 16: { using LL = CbLaunch<16>; return CALL; }     \
    case 32: { using LL = CbLaunch<32>; return CALL; }     \
    case 64: { using LL = CbLaunch<64>; return CALL; }     \
    case 128: { using LL = CbLaunch<128>; return CALL; }   \
    case 256: { using LL = CbLaunch<256>; return CALL; }   \
    case 512: { using LL = CbLaunch<512>; return CALL; }   \
    case 1024: { using LL = CbLaunch<1024>; return CALL; } \
    default: return cudaErrorInvalidValue;                 \
  }

cudaError_t cb_setup(int N) { SF21_CB_DISPATCH(N, LL::setup()); }
cudaError_t launch_rows_filter_cb(int N, const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st) {
  SF21_CB_DISPATCH(N, LL::rows(spec, bt, tw, st));
}
cudaError_t launch_cols_b_cb(int N, const Batch& bt, const float2* tw, cudaStream_t st) {
  SF21_CB_DISPATCH(N, LL::cols_b(bt, tw, st));
}
cudaError_t launch_cols_a_test_cb(int N, const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                                  cudaStream_t st) {
  SF21_CB_DISPATCH(N, LL::cols_a_test(bt, rc, alpha, tw, st));
}

}  // namespace sf21
