// Excursion-set halo finder on the GPU (get_halos.c:197-321).
//
// Filter bank: the z = 0 density spectrum F (one forward transform per box)
// is filtered for two masses at once, F (s W(k Ra) + i s W(k Rb)), s = dx^3 /
// L^3 growth, and inverted by one complex transform whose real and imaginary
// parts are the two filtered fields (F is Hermitian and W real, so both are
// real).  The a-axis inverse pass ends in the threshold of each field and
// writes one candidate bit per cell and mass (bit t of word t / 32 = cell t,
// t = (i N + j) N + p, the reference's scan order :236-239).  Two forms: over
// column-block-major work boxes (the production path) and over natural boxes
// (the field hook for the tests).
//
// Overlap test (:240-268), per mass in the reference's order: the reference
// accepts a candidate c when none of the cells of its sphere S(c) (the
// offsets of :244-257, a p-interval [-m, m] per (di, dj) row) is flagged,
// then flags all of them.  Same-mass candidates u < v conflict iff S(u) and
// S(v) share a cell, iff v - u lies in D = S + S (a p-interval of half-width
// m1 + m2 per row, maximised over the row splits).  The GPU form:
//   prefilter: a candidate whose sphere holds a flag of a larger mass is
//     rejected (flags only grow, so the reference rejects it too);
//   rounds: an undecided candidate with an accepted candidate in D is
//     rejected; one with no undecided candidate of lower index in D is
//     accepted.  Decisions read the bit sets of the previous round only, so
//     every decision is the sequential one (the lexicographically first
//     maximal independent set);
//   finisher: what the rounds leave undecided (long dependency chains, or
//     spheres too large for D) goes through the reference's loop in index
//     order on one CTA, the sphere's rows tested and set by all threads.
//     Candidates accepted by the rounds never conflict with an undecided one
//     of lower index, so their flags do not change its outcome.
// Flags are one bit per cell; rows of runs are tested and set word-wise.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cb_layout.cuh"
#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

// ---------------------------------------------------------------------------
// Filter bank
template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS)
k_hf_rows_filter(const float2* __restrict__ spec, HfBatch hb, const float2* __restrict__ gtw) {
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
  for (int k = 0; k < hb.K; ++k) {
    const HfPair& pr = hb.p[k];
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float wa = hb.scale * w_tophat(pr.dkRa * kmag[r]);
      const float wb = pr.bits_b ? hb.scale * w_tophat(pr.dkRb * kmag[r]) : 0.0f;
      v[r] = make_float2(z[r].x * wa - z[r].y * wb, z[r].x * wb + z[r].y * wa);
    }
    fft_line<N, true>(v, sbuf + row_in_cta * L::LS, stw, j);
    float2* dst = pr.work + row * N;
#pragma unroll
    for (int r = 0; r < 8; ++r) dst[j + r * (N / 8)] = v[r];
  }
}

// a-axis inverse + thresholds.  Lane layout of a warp: threadIdx = j CW + col,
// so one ballot covers 32 / CW rows of CW consecutive cells; the lane with
// col = 0 stores its row's CW bits (an aligned half-word or byte of the word).
template <int N>
__global__ void __launch_bounds__(ColGeom<N>::THREADS)
k_hf_cols_a_thresh(HfBatch hb, const float2* __restrict__ gtw) {
  using C = ColGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  load_twiddles<N>(stw, gtw);
  const int nblk = N / C::CW;
  const int b = blockIdx.x / nblk;
  const int c0 = (blockIdx.x % nblk) * C::CW;
  const long stride = (long)N * N;
  const long base = (long)b * N + c0;
  const int col = threadIdx.x % C::CW;
  const int j = threadIdx.x / C::CW;
  const int lane = threadIdx.x & 31;
  constexpr uint32_t cmask = (1u << C::CW) - 1u;
  for (int k = 0; k < hb.K; ++k) {
    const HfPair& pr = hb.p[k];
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = pr.work[base + (long)(j + r * (N / 8)) * stride + col];
    __syncthreads();
    fft_line<N, true>(v, sbuf + col * L::LS, stw, j);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const long t = base + (long)(j + r * (N / 8)) * stride;  // first cell of this row's CW cells
      const uint32_t ma = __ballot_sync(0xffffffffu, v[r].x > pr.thr_a);
      const uint32_t mb = __ballot_sync(0xffffffffu, v[r].y > pr.thr_b);
      if (col == 0) {
        if (C::CW == 16) {
          reinterpret_cast<uint16_t*>(pr.bits_a)[t >> 4] = (uint16_t)((ma >> lane) & cmask);
          if (pr.bits_b) reinterpret_cast<uint16_t*>(pr.bits_b)[t >> 4] = (uint16_t)((mb >> lane) & cmask);
        } else {
          reinterpret_cast<uint8_t*>(pr.bits_a)[t >> 3] = (uint8_t)((ma >> lane) & cmask);
          if (pr.bits_b) reinterpret_cast<uint8_t*>(pr.bits_b)[t >> 3] = (uint8_t)((mb >> lane) & cmask);
        }
      }
    }
    __syncthreads();
  }
}

// The same two passes over column-block-major work boxes (cb_layout.cuh),
// the production form: the c-axis pass writes each row as N / CW runs of CW
// values, the b-axis pass is kernels_cb.cu's k_cols_b_cb, and an a-axis tile
// (fixed b, one column block) reads N runs of CW values inside one slab.
template <int N>
__global__ void __launch_bounds__(CbGeom<N>::RTHREADS)
k_hf_rows_filter_cb(const float2* __restrict__ spec, HfBatch hb, const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using L = LineGeom<N>;
  constexpr int T = N / 8;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[2 * G::ROWS * L::LS];  // two exchange lines per row
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int row_in_cta = threadIdx.x / G::RT;
  const int j = threadIdx.x % G::RT;
  const long row = (long)blockIdx.x * G::ROWS + row_in_cta;
  const int a = (int)(row / N), b = (int)(row % N);
  float2* s0 = sbuf + row_in_cta * L::LS;
  float2* s1 = sbuf + (G::ROWS + row_in_cta) * L::LS;
  const int ka = kfreq(a, N), kb = kfreq(b, N);
  const int kab = ka * ka + kb * kb;
  float2 z[8];
  float kmag[8];
  const float2* src = spec + row * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int c = j + r * T;
    z[r] = __ldg(src + c);
    const int kc = kfreq(c, N);
    kmag[r] = sqrtf((float)(kab + kc * kc));
  }
  __syncthreads();
  for (int k = 0; k < hb.K; ++k) {
    const HfPair& pr = hb.p[k];
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float wa = hb.scale * w_tophat(pr.dkRa * kmag[r]);
      const float wb = pr.bits_b ? hb.scale * w_tophat(pr.dkRb * kmag[r]) : 0.0f;
      v[r] = make_float2(z[r].x * wa - z[r].y * wb, z[r].x * wb + z[r].y * wa);
    }
    if (FftPP<N>::CALL_SYNC) __syncthreads();
    fft_line_pp<N, true>(v, s0, s1, stw, j);
    if constexpr ((N / 8) % G::CW == 0) {
      float2* dst = pr.work + cb_index<N>(a, b, j);
      constexpr long RSTRIDE = (long)(N / 8 / G::CW) * N * N * G::CW;
#pragma unroll
      for (int r = 0; r < 8; ++r) dst[r * RSTRIDE] = v[r];
    } else {
#pragma unroll
      for (int r = 0; r < 8; ++r) pr.work[cb_index<N>(a, b, j + r * T)] = v[r];
    }
  }
}

template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, KGeom<N>::PER_SM)
k_hf_cols_a_thresh_cb(HfBatch hb, const float2* __restrict__ gtw) {
  using G = CbGeom<N>;
  using X = KGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const int lane = threadIdx.x & 31;
  // column block fastest: the NBLK tiles of one b write the neighbouring
  // half-words (bytes) of the same rows of the bit sets, so they run close
  // together and the L2 sectors fill before they are evicted (b fastest made
  // every bit-set store a read-modify-write of a sector from DRAM)
  const int cb = blockIdx.x % G::NBLK, b = blockIdx.x / G::NBLK;
  const long astride = (long)N * G::CW;
  const long tbase = ((long)cb * N * N + b) * G::CW + col;  // element (a = 0, b, cb CW + col)
  constexpr uint32_t cmask = (1u << G::CW) - 1u;
  auto load = [&](float2 (&v)[8], int k) {
    const float2* box = hb.p[k].work + tbase;
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = box[(long)(j + r * (N / 8)) * astride];
  };
  auto thresh = [&](const float2 (&v)[8], int k) {
    const HfPair& pr = hb.p[k];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const long t = ((long)(j + r * (N / 8)) * N + b) * N + (long)cb * G::CW;  // first cell of the run
      const uint32_t ma = __ballot_sync(0xffffffffu, v[r].x > pr.thr_a);
      const uint32_t mb = __ballot_sync(0xffffffffu, v[r].y > pr.thr_b);
      if (col == 0) {
        if (G::CW == 16) {
          reinterpret_cast<uint16_t*>(pr.bits_a)[t >> 4] = (uint16_t)((ma >> lane) & cmask);
          if (pr.bits_b) reinterpret_cast<uint16_t*>(pr.bits_b)[t >> 4] = (uint16_t)((mb >> lane) & cmask);
        } else {
          reinterpret_cast<uint8_t*>(pr.bits_a)[t >> 3] = (uint8_t)((ma >> lane) & cmask);
          if (pr.bits_b) reinterpret_cast<uint8_t*>(pr.bits_b)[t >> 3] = (uint8_t)((mb >> lane) & cmask);
        }
      }
    }
  };
  float2* s0 = sbuf + col * X::LS;
  float2* s1 = sbuf + (X::KW + col) * X::LS;
  float2 va[8], vb[8];
  load(va, 0);
  __syncthreads();  // twiddles
  for (int k = 0; k < hb.K; k += 2) {
    if (k + 1 < hb.K) load(vb, k + 1);
    if (FftPP<N>::CALL_SYNC && k > 0) __syncthreads();
    fft_line_pp<N, true>(va, s0, s1, stw, j);
    thresh(va, k);
    if (k + 1 < hb.K) {
      if (k + 2 < hb.K) load(va, k + 2);
      if (FftPP<N>::CALL_SYNC) __syncthreads();
      fft_line_pp<N, true>(vb, s0, s1, stw, j);
      thresh(vb, k + 1);
    }
  }
}

template <int N>
struct HfLaunch {
  static constexpr size_t smem_cols() { return (N + ColGeom<N>::CW * LineGeom<N>::LS) * sizeof(float2); }
  static cudaError_t rows(const float2* spec, const HfBatch& hb, const float2* tw, cudaStream_t st) {
    k_hf_rows_filter<N><<<(unsigned)((long)N * N / RowGeom<N>::ROWS), RowGeom<N>::THREADS, 0, st>>>(spec, hb, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols_a(const HfBatch& hb, const float2* tw, cudaStream_t st) {
    k_hf_cols_a_thresh<N><<<(unsigned)((long)N * (N / ColGeom<N>::CW)), ColGeom<N>::THREADS, smem_cols(), st>>>(hb,
                                                                                                               tw);
    return cudaGetLastError();
  }
  static cudaError_t rows_cb(const float2* spec, const HfBatch& hb, const float2* tw, cudaStream_t st) {
    using G = CbGeom<N>;
    k_hf_rows_filter_cb<N><<<(unsigned)((long)N * N / G::ROWS), G::RTHREADS, 0, st>>>(spec, hb, tw);
    return cudaGetLastError();
  }
  static cudaError_t cols_a_cb(const HfBatch& hb, const float2* tw, cudaStream_t st) {
    using X = KGeom<N>;
    k_hf_cols_a_thresh_cb<N><<<(unsigned)(N * CbGeom<N>::NBLK), X::THREADS, X::SMEM, st>>>(hb, tw);
    return cudaGetLastError();
  }
  static cudaError_t setup() {
    cudaError_t e = cudaFuncSetAttribute(k_hf_cols_a_thresh<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_cols());
    if (e) return e;
    return cudaFuncSetAttribute(k_hf_cols_a_thresh_cb<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)KGeom<N>::SMEM);
  }
};

#define SF21_HF_DISPATCH(N, CALL)                         \
  switch (N) {                                            \
    case 16: { using HL = HfLaunch<16>; return CALL; }    \
    case 32: { using HL = HfLaunch<32>; return CALL; }    \
    case 64: { using HL = HfLaunch<64>; return CALL; }    \
    case 128: { using HL = HfLaunch<128>; return CALL; }  \
    case 256: { using HL = HfLaunch<256>; return CALL; }  \
    case 512: { using HL = HfLaunch<512>; return CALL; }  \
    case 1024: { using HL = HfLaunch<1024>; return CALL; } \
    default: return cudaErrorInvalidValue;                \
  }

cudaError_t hf_setup(int N) { SF21_HF_DISPATCH(N, HL::setup()); }
cudaError_t launch_hf_rows_filter(int N, const float2* spec, const HfBatch& hb, const float2* tw, cudaStream_t st) {
  SF21_HF_DISPATCH(N, HL::rows(spec, hb, tw, st));
}
cudaError_t launch_hf_cols_a_thresh(int N, const HfBatch& hb, const float2* tw, cudaStream_t st) {
  SF21_HF_DISPATCH(N, HL::cols_a(hb, tw, st));
}
cudaError_t launch_hf_rows_filter_cb(int N, const float2* spec, const HfBatch& hb, const float2* tw,
                                     cudaStream_t st) {
  SF21_HF_DISPATCH(N, HL::rows_cb(spec, hb, tw, st));
}
cudaError_t launch_hf_cols_a_thresh_cb(int N, const HfBatch& hb, const float2* tw, cudaStream_t st) {
  SF21_HF_DISPATCH(N, HL::cols_a_cb(hb, tw, st));
}

// ---------------------------------------------------------------------------
// Bit sets
__device__ __forceinline__ uint32_t ldw(const uint32_t* W, long w) { return __ldcg(W + w); }

// any set bit in the inclusive range [b0, b1]
__device__ bool bits_any(const uint32_t* W, long b0, long b1) {
  if (b0 > b1) return false;
  const long w0 = b0 >> 5, w1 = b1 >> 5;
  const uint32_t m0 = 0xffffffffu << (b0 & 31);
  const uint32_t m1 = 0xffffffffu >> (31 - (b1 & 31));
  if (w0 == w1) return (ldw(W, w0) & m0 & m1) != 0;
  if (ldw(W, w0) & m0) return true;
  for (long w = w0 + 1; w < w1; ++w)
    if (ldw(W, w)) return true;
  return (ldw(W, w1) & m1) != 0;
}

__device__ void bits_set(uint32_t* W, long b0, long b1) {
  if (b0 > b1) return;
  const long w0 = b0 >> 5, w1 = b1 >> 5;
  const uint32_t m0 = 0xffffffffu << (b0 & 31);
  const uint32_t m1 = 0xffffffffu >> (31 - (b1 & 31));
  if (w0 == w1) {
    atomicOr(W + w0, m0 & m1);
    return;
  }
  atomicOr(W + w0, m0);
  for (long w = w0 + 1; w < w1; ++w) atomicOr(W + w, 0xffffffffu);
  atomicOr(W + w1, m1);
}

// The run of row (a, b) over p - m .. p + m (periodic in p) as at most two
// inclusive bit ranges; a range with r0 > r1 is empty.
struct RunBits {
  long r0, r1, s0, s1;
};
__device__ __forceinline__ RunBits run_bits(int N, long row, int p, int m) {
  const long base = row * N;
  RunBits rb;
  rb.s0 = 1;
  rb.s1 = 0;
  if (2 * m + 1 >= N) {
    rb.r0 = base;
    rb.r1 = base + N - 1;
    return rb;
  }
  const int lo = p - m, hi = p + m;
  if (lo < 0) {
    rb.r0 = base;
    rb.r1 = base + hi;
    rb.s0 = base + lo + N;
    rb.s1 = base + N - 1;
  } else if (hi >= N) {
    rb.r0 = base + lo;
    rb.r1 = base + N - 1;
    rb.s0 = base;
    rb.s1 = base + hi - N;
  } else {
    rb.r0 = base + lo;
    rb.r1 = base + hi;
  }
  return rb;
}

__device__ __forceinline__ int wrapi(int x, int N) { return x < 0 ? x + N : (x >= N ? x - N : x); }

struct Cell {
  int i, j, p;
};
__device__ __forceinline__ Cell decode(uint32_t u, int N) {
  Cell c;
  const uint32_t q = u / (uint32_t)N;
  c.p = (int)(u - q * (uint32_t)N);
  c.i = (int)(q / (uint32_t)N);
  c.j = (int)(q - (uint32_t)c.i * (uint32_t)N);
  return c;
}

__device__ __forceinline__ long run_row(const Cell& c, int4 q, int N) {
  return (long)wrapi(c.i + q.x, N) * N + wrapi(c.j + q.y, N);
}

__device__ __forceinline__ bool run_any(const uint32_t* W, int N, const Cell& c, int4 q) {
  const RunBits rb = run_bits(N, run_row(c, q, N), c.p, q.z);
  return bits_any(W, rb.r0, rb.r1) || bits_any(W, rb.s0, rb.s1);
}

// only bits of index < lim
__device__ __forceinline__ bool run_any_below(const uint32_t* W, int N, const Cell& c, int4 q, long lim) {
  const RunBits rb = run_bits(N, run_row(c, q, N), c.p, q.z);
  return bits_any(W, rb.r0, rb.r1 < lim ? rb.r1 : lim - 1) || bits_any(W, rb.s0, rb.s1 < lim ? rb.s1 : lim - 1);
}

__device__ __forceinline__ void run_set(uint32_t* W, int N, const Cell& c, int4 q) {
  const RunBits rb = run_bits(N, run_row(c, q, N), c.p, q.z);
  bits_set(W, rb.r0, rb.r1);
  bits_set(W, rb.s0, rb.s1);
}

// ---------------------------------------------------------------------------
// Compaction of a bit set into the sorted list of its set positions.
constexpr int CMP_THREADS = 256;
constexpr int CMP_WPT = 32;                             // words per thread
constexpr long CMP_CHUNK = (long)CMP_THREADS * CMP_WPT;  // words per CTA

long hf_compact_chunks(long nwords) { return (nwords + CMP_CHUNK - 1) / CMP_CHUNK; }

__global__ void __launch_bounds__(CMP_THREADS) k_bits_count(const uint32_t* __restrict__ W, long nwords,
                                                            uint32_t* __restrict__ cnt) {
  const long w0 = blockIdx.x * CMP_CHUNK;
  uint32_t s = 0;
  for (long w = w0 + threadIdx.x; w < w0 + CMP_CHUNK && w < nwords; w += CMP_THREADS) s += __popc(W[w]);
  s = __reduce_add_sync(0xffffffffu, s);
  __shared__ uint32_t red[CMP_THREADS / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int k = 0; k < CMP_THREADS / 32; ++k) t += red[k];
    cnt[blockIdx.x] = t;
  }
}

// exclusive scan of n counts in place (one CTA of 1024 threads); total -> *tot
__global__ void __launch_bounds__(1024) k_scan_counts(uint32_t* __restrict__ cnt, long n, uint32_t* __restrict__ tot) {
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long base = 0; base < n; base += 1024) {
    const long t = base + threadIdx.x;
    const uint32_t v = t < n ? cnt[t] : 0u;
    uint32_t x = v;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      uint32_t s = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      wsum[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t excl = carry + (w ? wsum[w - 1] : 0u) + x - v;
    if (t < n) cnt[t] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *tot = carry;
}

__global__ void __launch_bounds__(CMP_THREADS) k_bits_emit(const uint32_t* __restrict__ W, long nwords,
                                                           const uint32_t* __restrict__ off,
                                                           uint32_t* __restrict__ out) {
  // thread t owns words w0 + t*CMP_WPT .. +CMP_WPT-1 (contiguous, keeps order)
  const long w0 = blockIdx.x * CMP_CHUNK + (long)threadIdx.x * CMP_WPT;
  uint32_t s = 0;
  for (int k = 0; k < CMP_WPT; ++k)
    if (w0 + k < nwords) s += __popc(__ldg(W + w0 + k));
  // block exclusive scan of s
  __shared__ uint32_t wsum[CMP_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int k = 0; k < w; ++k) before += wsum[k];
  uint32_t pos = off[blockIdx.x] + before + x - s;
  for (int k = 0; k < CMP_WPT; ++k) {
    const long wi = w0 + k;
    if (wi >= nwords) break;
    uint32_t m = __ldg(W + wi);
    while (m) {
      const int bit = __ffs(m) - 1;
      out[pos++] = (uint32_t)(wi * 32 + bit);
      m &= m - 1;
    }
  }
}

cudaError_t launch_bits_count(const uint32_t* W, long nwords, uint32_t* cnt, cudaStream_t st) {
  k_bits_count<<<(unsigned)hf_compact_chunks(nwords), CMP_THREADS, 0, st>>>(W, nwords, cnt);
  return cudaGetLastError();
}
cudaError_t launch_scan_counts(uint32_t* cnt, long n, uint32_t* tot, cudaStream_t st) {
  k_scan_counts<<<1, 1024, 0, st>>>(cnt, n, tot);
  return cudaGetLastError();
}
cudaError_t launch_bits_emit(const uint32_t* W, long nwords, const uint32_t* off, uint32_t* out, cudaStream_t st) {
  k_bits_emit<<<(unsigned)hf_compact_chunks(nwords), CMP_THREADS, 0, st>>>(W, nwords, off, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Overlap test
constexpr int GL_THREADS = 256;
static unsigned gl_grid() { return 152 * 8; }

__device__ __forceinline__ long warp_id_global() { return ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ long warps_total() { return ((long)gridDim.x * blockDim.x) >> 5; }

__global__ void __launch_bounds__(GL_THREADS)
k_hf_prefilter(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_ptr, int N,
               const int4* __restrict__ runs, int nruns, const uint32_t* __restrict__ FL, uint32_t* __restrict__ UND,
               uint8_t* __restrict__ status, uint32_t* __restrict__ n_und) {
  const long n = *n_ptr;
  const int lane = threadIdx.x & 31;
  for (long c = warp_id_global(); c < n; c += warps_total()) {
    const uint32_t u = list[c];
    const Cell cl = decode(u, N);
    bool hit = false;
    for (int r0 = 0; r0 < nruns && !hit; r0 += 32) {
      const int r = r0 + lane;
      const bool h = r < nruns && run_any(FL, N, cl, runs[r]);
      hit = __any_sync(0xffffffffu, h);
    }
    if (lane == 0) {
      status[c] = hit ? HF_REJ : HF_UND;
      if (!hit) {
        atomicOr(UND + (u >> 5), 1u << (u & 31));
        atomicAdd(n_und, 1u);
      }
    }
  }
}

__global__ void __launch_bounds__(GL_THREADS)
k_hf_round_decide(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_ptr, int N,
                  const int4* __restrict__ druns, int ndruns, const uint32_t* __restrict__ UND,
                  const uint32_t* __restrict__ ACC, uint8_t* __restrict__ status,
                  const uint32_t* __restrict__ n_und) {
  if (*n_und == 0) return;
  const long n = *n_ptr;
  const int lane = threadIdx.x & 31;
  for (long c = warp_id_global(); c < n; c += warps_total()) {
    if (status[c] != HF_UND) continue;
    const uint32_t u = list[c];
    const Cell cl = decode(u, N);
    bool acc = false, earlier = false;
    for (int r0 = 0; r0 < ndruns && !acc; r0 += 32) {
      const int r = r0 + lane;
      bool a = false, e = false;
      if (r < ndruns) {
        const int4 q = druns[r];
        a = run_any(ACC, N, cl, q);
        e = !a && !earlier && run_any_below(UND, N, cl, q, (long)u);
      }
      acc = __any_sync(0xffffffffu, a);
      earlier = __any_sync(0xffffffffu, e) || earlier;
    }
    if (lane == 0) {
      if (acc)
        status[c] = HF_PEND_REJ;
      else if (!earlier)
        status[c] = HF_PEND_ACC;
    }
  }
}

__global__ void __launch_bounds__(GL_THREADS)
k_hf_round_apply(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_ptr, uint32_t* __restrict__ UND,
                 uint32_t* __restrict__ ACC, uint8_t* __restrict__ status, uint32_t* __restrict__ n_und) {
  if (*n_und == 0) return;
  const long n = *n_ptr;
  uint32_t done = 0;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
    const uint8_t s = status[c];
    if (s != HF_PEND_ACC && s != HF_PEND_REJ) continue;
    const uint32_t u = list[c];
    atomicAnd(UND + (u >> 5), ~(1u << (u & 31)));
    if (s == HF_PEND_ACC) {
      atomicOr(ACC + (u >> 5), 1u << (u & 31));
      status[c] = HF_ACC;
    } else {
      status[c] = HF_REJ;
    }
    ++done;
  }
  done = __reduce_add_sync(0xffffffffu, done);
  if ((threadIdx.x & 31) == 0 && done) atomicSub(n_und, done);
}

// Flag the spheres of candidates accepted by the rounds (status HF_ACC).
__global__ void __launch_bounds__(GL_THREADS)
k_hf_flag_accepted(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_ptr, int N,
                   const int4* __restrict__ runs, int nruns, uint32_t* __restrict__ FL, uint8_t* __restrict__ status) {
  const long n = *n_ptr;
  const int lane = threadIdx.x & 31;
  for (long c = warp_id_global(); c < n; c += warps_total()) {
    if (status[c] != HF_ACC) continue;
    const Cell cl = decode(list[c], N);
    for (int r = lane; r < nruns; r += 32) run_set(FL, N, cl, runs[r]);
    __syncwarp();
    if (lane == 0) status[c] = HF_ACC_FLAGGED;
  }
}

// The reference's loop (:236-279) over the still-undecided candidates, in
// index order, on one CTA.
constexpr int FIN_THREADS = 1024;
__global__ void __launch_bounds__(FIN_THREADS)
k_hf_finisher(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_ptr, int N,
              const int4* __restrict__ runs, int nruns, uint32_t* __restrict__ FL, uint32_t* __restrict__ ACC,
              uint8_t* __restrict__ status) {
  const long n = *n_ptr;
  __shared__ uint32_t todo[FIN_THREADS];
  __shared__ int ntodo;
  __shared__ int wcnt[FIN_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (long c0 = 0; c0 < n; c0 += FIN_THREADS) {
    const long c = c0 + threadIdx.x;
    const bool und = c < n && status[c] == HF_UND;
    // ordered list of the chunk's undecided entries
    const uint32_t bal = __ballot_sync(0xffffffffu, und);
    if (lane == 0) wcnt[w] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = 0;
      for (int k = 0; k < FIN_THREADS / 32; ++k) {
        const int t = wcnt[k];
        wcnt[k] = s;
        s += t;
      }
      ntodo = s;
    }
    __syncthreads();
    if (und) todo[wcnt[w] + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)threadIdx.x;
    __syncthreads();
    const int nt = ntodo;
    for (int k = 0; k < nt; ++k) {
      const long ck = c0 + todo[k];
      const Cell cl = decode(list[ck], N);
      bool h = false;
      for (int r = threadIdx.x; r < nruns && !h; r += FIN_THREADS) h = run_any(FL, N, cl, runs[r]);
      const int hit = __syncthreads_or(h);
      if (!hit) {
        for (int r = threadIdx.x; r < nruns; r += FIN_THREADS) run_set(FL, N, cl, runs[r]);
        if (threadIdx.x == 0) {
          const uint32_t u = list[ck];
          atomicOr(ACC + (u >> 5), 1u << (u & 31));
          status[ck] = HF_ACC_FLAGGED;
        }
      } else if (threadIdx.x == 0) {
        status[ck] = HF_REJ;
      }
      __threadfence();
      __syncthreads();
    }
  }
}

// Clear the candidates' bits in UND and ACC (ready for the next mass).
__global__ void k_hf_clear(const uint32_t* __restrict__ list, const uint32_t* __restrict__ n_ptr,
                           uint32_t* __restrict__ UND, uint32_t* __restrict__ ACC) {
  const long n = *n_ptr;
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
    const uint32_t u = list[c];
    const uint32_t m = ~(1u << (u & 31));
    atomicAnd(UND + (u >> 5), m);
    atomicAnd(ACC + (u >> 5), m);
  }
}

// Cell-size cycle (:293-321): cell t is a halo when unflagged and
// delta_z0 * growth > deltaCMZ, which for floats is delta_z0 >= tcell (the
// threshold found on the host).  Flags the cells found.  One warp per 32
// words, lane k keeps word k.
__global__ void k_hf_cell(long nwords, const float* __restrict__ delta, float tcell, uint32_t* __restrict__ FL,
                          uint32_t* __restrict__ bits) {
  const int lane = threadIdx.x & 31;
  for (long w0 = warp_id_global() * 32; w0 < nwords; w0 += warps_total() * 32) {
    uint32_t mine = 0;
    for (int k = 0; k < 32; ++k) {
      const long w = w0 + k;
      if (w >= nwords) break;
      const uint32_t m = __ballot_sync(0xffffffffu, delta[w * 32 + lane] >= tcell);
      if (lane == k) mine = m;
    }
    const long w = w0 + lane;
    if (w < nwords) {
      const uint32_t f = FL[w];
      const uint32_t cell = mine & ~f;
      bits[w] = cell;
      FL[w] = f | cell;
    }
  }
}

// Catalogue records {Mass, x, y, z} (Halo_t, auxiliary.h:13-17) of a sorted
// cell list.
__global__ void k_hf_records(const uint32_t* __restrict__ idx, long n, int N, float mass,
                             float4* __restrict__ out) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const Cell c = decode(idx[k], N);
    out[k] = make_float4(mass, (float)c.i, (float)c.j, (float)c.p);
  }
}

cudaError_t launch_hf_prefilter(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* runs, int nruns,
                                const uint32_t* FL, uint32_t* UND, uint8_t* status, uint32_t* n_und,
                                cudaStream_t st) {
  k_hf_prefilter<<<gl_grid(), GL_THREADS, 0, st>>>(list, n_ptr, N, runs, nruns, FL, UND, status, n_und);
  return cudaGetLastError();
}
cudaError_t launch_hf_round(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* druns, int ndruns,
                            uint32_t* UND, uint32_t* ACC, uint8_t* status, uint32_t* n_und, cudaStream_t st) {
  k_hf_round_decide<<<gl_grid(), GL_THREADS, 0, st>>>(list, n_ptr, N, druns, ndruns, UND, ACC, status, n_und);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  k_hf_round_apply<<<gl_grid(), GL_THREADS, 0, st>>>(list, n_ptr, UND, ACC, status, n_und);
  return cudaGetLastError();
}
cudaError_t launch_hf_flag_accepted(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* runs,
                                    int nruns, uint32_t* FL, uint8_t* status, cudaStream_t st) {
  k_hf_flag_accepted<<<gl_grid(), GL_THREADS, 0, st>>>(list, n_ptr, N, runs, nruns, FL, status);
  return cudaGetLastError();
}
cudaError_t launch_hf_finisher(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* runs, int nruns,
                               uint32_t* FL, uint32_t* ACC, uint8_t* status, cudaStream_t st) {
  k_hf_finisher<<<1, FIN_THREADS, 0, st>>>(list, n_ptr, N, runs, nruns, FL, ACC, status);
  return cudaGetLastError();
}
cudaError_t launch_hf_clear(const uint32_t* list, const uint32_t* n_ptr, uint32_t* UND, uint32_t* ACC,
                            cudaStream_t st) {
  k_hf_clear<<<gl_grid(), GL_THREADS, 0, st>>>(list, n_ptr, UND, ACC);
  return cudaGetLastError();
}
cudaError_t launch_hf_cell(long nwords, const float* delta, float tcell, uint32_t* FL, uint32_t* bits,
                           cudaStream_t st) {
  k_hf_cell<<<gl_grid(), GL_THREADS, 0, st>>>(nwords, delta, tcell, FL, bits);
  return cudaGetLastError();
}
cudaError_t launch_hf_records(const uint32_t* idx, long n, int N, float mass, float4* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  k_hf_records<<<(unsigned)b, 256, 0, st>>>(idx, n, N, mass, out);
  return cudaGetLastError();
}

}  // namespace sf21
