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

#include "cb_layout.cuh"
#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

// c-axis inverse pass with the top-hat filter of the K radii of the batch
// (get_HIIbubbles.c:305-322): spectrum row (a, b) read once, K filtered
// transformed rows written column-block major.  One row per T = N/8 threads
// (j = thread index in the row, s0/s1 = this row's two exchange lines).
// (Sharing the N/2 + 1 distinct window values of a row through shared memory
// or warp shuffles measured slower than evaluating W per element.)
template <int N>
__device__ __forceinline__ void rows_filter_row(const float2* __restrict__ spec, const Batch& bt,
                                                const float2* stw, float2* s0, float2* s1, int a, int b, int j) {
  using G = CbGeom<N>;
  constexpr int T = N / 8;
  const int ka = kfreq(a, N), kb = kfreq(b, N);
  const int kab = ka * ka + kb * kb;
  float2 z[8];
  float kmag[8];
  const float2* src = spec + ((long)a * N + b) * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int c = j + r * T;
    z[r] = __ldg(src + c);
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
    if (FftPP<N>::CALL_SYNC) __syncthreads();
    fft_line_pp<N, true>(v, s0, s1, stw, j);
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

template <int N>
__global__ void __launch_bounds__(CbGeom<N>::RTHREADS)
k_rows_filter_cb(const float2* __restrict__ spec, Batch bt, const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using L = LineGeom<N>;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[2 * G::ROWS * L::LS];  // two exchange lines per row
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int row_in_cta = threadIdx.x / G::RT;
  const int j = threadIdx.x % G::RT;
  const long row = (long)blockIdx.x * G::ROWS + row_in_cta;
  rows_filter_row<N>(spec, bt, stw, sbuf + row_in_cta * L::LS, sbuf + (G::ROWS + row_in_cta) * L::LS,
                     (int)(row / N), (int)(row % N), j);
}

// b-axis inverse pass in place: tile (a, column block) = one contiguous run
// of N CW values per radius.  One CTA per tile (blockIdx.x = cb N + a) walks
// the K radii with two register sets in turn, the loads of radius k + 1 in
// flight during the transform of radius k.  (A persistent form with
// prefetch across tiles, as in the a-axis pass below, measured 5 % slower
// here: this pass is at the HBM roofline and the hardware's dynamic tile
// order keeps the concurrent tiles' accesses closer together.)
//
// A CTA takes the whole column block: with 16 columns a warp covers 16
// lines x 2 threads, whose shared-memory exchanges of the line FFT are free of
// bank conflicts.  (Half blocks of 8 columns, two CTAs per SM, measured
// slower even with a conflict-free exchange padding.)
template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, KGeom<N>::PER_SM)
k_cols_b_cb(Batch bt, const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using X = KGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const long off = (long)blockIdx.x * N * G::CW + col;  // element (b = 0) of this column
  auto load = [&](float2 (&v)[8], int k) {
    const float2* box = bt.r[k].work + off;
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = box[(j + r * (N / 8)) * G::CW];
  };
  auto store = [&](const float2 (&v)[8], int k) {
    float2* box = bt.r[k].work + off;
#pragma unroll
    for (int r = 0; r < 8; ++r) box[(j + r * (N / 8)) * G::CW] = v[r];
  };
  float2* s0 = sbuf + col * X::LS;
  float2* s1 = sbuf + (X::KW + col) * X::LS;
  float2 va[8], vb[8];
  load(va, 0);
  __syncthreads();  // twiddles
  for (int k = 0; k < bt.K; k += 2) {
    if (k + 1 < bt.K) load(vb, k + 1);
    if (FftPP<N>::CALL_SYNC && k > 0) __syncthreads();
    fft_line_pp<N, true>(va, s0, s1, stw, j);
    store(va, k);
    if (k + 1 < bt.K) {
      if (k + 2 < bt.K) load(va, k + 2);
      if (FftPP<N>::CALL_SYNC) __syncthreads();
      fft_line_pp<N, true>(vb, s0, s1, stw, j);
      store(vb, k + 1);
    }
  }
}

// a-axis inverse pass of the K radii + centre test + first-hit update
// (get_HIIbubbles.c:335-352; centre test: is_centre).  Persistent (5 %
// faster here than one CTA per tile): CTA i
// takes tiles i, i + gridDim.x, ... (tile = cb N + b: one column block of
// one b) and walks each tile's K radii.  The steps (tile, radius) use two
// register sets in turn and the loads of the next step -- the next radius,
// or radius 0 of the next tile -- are issued before the transform of the
// current one, so every warp keeps a tile in flight while it computes, also
// across tiles.
template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, KGeom<N>::PER_SM)
k_cols_a_test_cb(Batch bt, uint8_t* __restrict__ rc, const float* __restrict__ alpha_ptr,
                 const float2* __restrict__ gtw, int ntiles) {
  using G = CbGeom<N>;
  using X = KGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const float alpha = *alpha_ptr;
  const float zmul = bt.zmul;
  const int K = bt.K;
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const long astride = (long)N * G::CW;
  // element (a = 0, b, cb CW + col) of tile cb N + b
  auto tile_base = [&](int tile) { return ((long)(tile / N) * N * N + tile % N) * G::CW + col; };
  // bit 8 (r & 3) + k of m[r / 4]: element r is a centre at radius k of the
  // batch (radius indices increase with k, so the lowest bit is the first hit)
  uint32_t m[2] = {0u, 0u};
  auto test = [&](const float2 (&v)[8], int k) {
    const uint32_t bit = 1u << k;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (is_centre(v[r], alpha, zmul)) m[r >> 2] |= bit << (8 * (r & 3));
    }
  };
  auto load = [&](float2 (&v)[8], int tile, int k) {
    const float2* box = bt.r[k].work + tile_base(tile);
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = box[(long)(j + r * (N / 8)) * astride];
  };
  auto flush = [&](int tile) {  // first-hit update of the tile, once per tile
    const int b = tile % N;
    const int c = (tile / N) * G::CW + col;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const uint32_t byte = (m[r >> 2] >> (8 * (r & 3))) & 0xFFu;
      if (byte) {
        const uint32_t h = (uint32_t)bt.r[__ffs(byte) - 1].ridx;
        const long idx = ((long)(j + r * (N / 8)) * N + b) * N + c;
        const uint8_t old = rc[idx];
        if (h < old) rc[idx] = (uint8_t)h;
      }
    }
    m[0] = m[1] = 0u;
  };
  float2* s0 = sbuf + col * X::LS;
  float2* s1 = sbuf + (X::KW + col) * X::LS;
  int tile = blockIdx.x, k = 0;
  if (tile >= ntiles) return;
  float2 va[8], vb[8];
  load(va, tile, 0);
  __syncthreads();  // twiddles
  for (bool first = true;; first = false) {
    // step (tile, k) in va; the next step goes to vb
    int kb = k + 1, tb = tile;
    if (kb == K) { kb = 0; tb += gridDim.x; }
    const bool has_b = tb < ntiles;
    if (has_b) load(vb, tb, kb);
    if (FftPP<N>::CALL_SYNC && !first) __syncthreads();
    fft_line_pp<N, true>(va, s0, s1, stw, j);
    test(va, k);
    if (k == K - 1) flush(tile);
    if (!has_b) break;
    // step (tb, kb) in vb; the next step goes to va
    int kc = kb + 1, tc = tb;
    if (kc == K) { kc = 0; tc += gridDim.x; }
    const bool has_c = tc < ntiles;
    if (has_c) load(va, tc, kc);
    if (FftPP<N>::CALL_SYNC) __syncthreads();
    fft_line_pp<N, true>(vb, s0, s1, stw, j);
    test(vb, kb);
    if (kb == K - 1) flush(tb);
    if (!has_c) break;
    tile = tc;
    k = kc;
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
  static int grid(int nsm) {
    const int ntiles = N * G::NBLK;
    return ntiles < nsm * KGeom<N>::PER_SM ? ntiles : nsm * KGeom<N>::PER_SM;
  }
  static cudaError_t cols_b(const Batch& bt, const float2* tw, cudaStream_t st) {
    using X = KGeom<N>;
    k_cols_b_cb<N><<<(unsigned)(N * G::NBLK), X::THREADS, X::SMEM, st>>>(bt, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols_a_test(const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw, int nsm,
                                 cudaStream_t st) {
    using X = KGeom<N>;
    k_cols_a_test_cb<N><<<grid(nsm), X::THREADS, X::SMEM, st>>>(bt, rc, alpha, tw, N * G::NBLK);
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
cudaError_t launch_cols_a_test_cb(int N, const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw, int nsm,
                                  cudaStream_t st) {
  SF21_CB_DISPATCH(N, LL::cols_a_test(bt, rc, alpha, tw, nsm, st));
}

}  // namespace sf21
