// b- and a-axis inverse passes of a batch in one persistent launch, the
// b-axis output handed to the a-axis pass through L2 (radius pipeline 8).
//
// In the column-block-major work layout (kernels_cb.cu) the b- and a-axis
// transforms of one radius touch one column block's slab of N^2 CW values
// (32 MB at N = 512) and nothing else.  The launch walks the slabs ("units",
// u = k NBLK + cb for radius k of the batch and column block cb) in order and
// interleaves, tile by tile, the b-axis tiles of unit u (fixed a: one
// contiguous N CW run, transformed in place) with the a-axis tiles of unit
// u - 1 (fixed b: N runs of CW values N CW apart; transform, centre test,
// first-hit update).  So about two slabs are live at a time, which L2 holds:
// the a-axis pass reads the b-axis output from L2 (ld.global.cg), and once a
// tile's lines have been read they are dropped from L2 without a write-back
// (discard.global.L2: the values are dead).  Per voxel and radius the DRAM
// sees the c-axis pass's write and the b-axis pass's read, the north-star
// "one HBM round trip per radius", instead of two.
//
// Work queue: one CTA per SM takes queue positions from an atomic counter in
// a fixed order.  An a-axis tile of unit u waits until all N b-axis tiles of
// u have published (per-unit counter; release by threadfence + atomic,
// acquire load), and until the a-axis tiles of unit u - NBLK (the same
// column block at the previous radius) have finished, so that the first-hit
// updates of one voxel happen in radius order (no read-modify-write race on
// rc).  b-axis tiles never wait, and every tile a CTA waits for sits earlier
// in the queue and is held by a running CTA, so the launch always completes.
// The next position's loads are issued before the current tile is
// transformed when they need no wait (always for b-axis tiles; for a-axis
// tiles when their units are already done, the common case: the b-axis
// tiles of unit u are a whole unit ahead in the queue).
//
// Every wait is bounded (spin_limit polls): on expiry the CTA records the
// error in *err and carries on, and the host reports SF21_E_TIMEOUT.
//
// ctl (ints, zeroed before each launch): [0] queue head, [1 + u] b-axis tiles
// done in unit u, [1 + U + u] a-axis tiles done in unit u (U = K NBLK).
#include <cuda_runtime.h>
#include <stdint.h>

#include "cb_layout.cuh"
#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

#define SF21_FUSED_SPIN_LIMIT (1u << 26)

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void discard_l2_line(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

// Queue position p -> (kind 0 = b-axis tile, 1 = a-axis tile, unit, tile).
template <int N>
__device__ __forceinline__ void fused_decode(long p, int U, int& kind, int& u, int& t) {
  const long lead = N;
  const long mid = 2L * N * (U - 1);
  if (p < lead) {
    kind = 0;
    u = 0;
    t = (int)p;
  } else if (p < lead + mid) {
    const long q = p - lead;
    const long seg = q / (2 * N), w = q % (2 * N);
    t = (int)(w >> 1);
    kind = (int)(w & 1);
    u = kind ? (int)seg : (int)seg + 1;
  } else {
    kind = 1;
    u = U - 1;
    t = (int)(p - lead - mid);
  }
}

template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, 1)
k_cols_ba_fused(Batch bt, uint8_t* __restrict__ rc, const float* __restrict__ alpha_ptr,
                const float2* __restrict__ gtw, int* ctl, int* __restrict__ err, uint32_t spin_limit) {
  using G = CbGeom<N>;
  using X = KGeom<N>;
  constexpr int CW = G::CW;
  constexpr int NBLK = G::NBLK;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  __shared__ long s_pos[2];
  __shared__ int s_ready[2];
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const float alpha = *alpha_ptr;
  const float zmul = bt.zmul;
  const int U = bt.K * NBLK;
  const long total = 2L * N * U;
  int* head = ctl;
  int* ky_done = ctl + 1;
  int* kx_done = ctl + 1 + U;
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const long astride = (long)N * CW;
  float2* s0 = sbuf + col * X::LS;
  float2* s1 = sbuf + (X::KW + col) * X::LS;

  // dependencies of an a-axis tile of unit u are met
  auto deps_met = [&](int u) {
    if (ld_acquire_gpu(ky_done + u) < N) return false;
    return u < NBLK || ld_acquire_gpu(kx_done + u - NBLK) >= N;
  };
  auto wait_deps = [&](int u) {  // thread 0 only
    for (uint32_t it = 0; it < spin_limit; ++it) {
      if (deps_met(u)) return;
      __nanosleep(64);
    }
    atomicExch(err, 2);
  };
  // element (row 0) of this thread's column in tile t of unit u
  auto tile_ptr = [&](int kind, int u, int t) -> float2* {
    const int k = u / NBLK, cb = u % NBLK;
    float2* box = bt.r[k].work;
    return kind == 0 ? box + ((long)cb * N + t) * N * CW + col : box + ((long)cb * N * N + t) * CW + col;
  };
  auto load = [&](float2 (&v)[8], int kind, int u, int t) {
    const float2* p = tile_ptr(kind, u, t);
    if (kind == 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = p[(j + r * (N / 8)) * CW];
    } else {
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = __ldcg(p + (long)(j + r * (N / 8)) * astride);
    }
  };

  // position pos is taken by thread 0 into s_pos[b]; s_ready[b] = 1 when its
  // loads may be issued now (no wait needed)
  auto fetch = [&](int b) {
    const long p = atomicAdd(head, 1);
    s_pos[b] = p;
    int ready = 1;
    if (p < total) {
      int kind, u, t;
      fused_decode<N>(p, U, kind, u, t);
      if (kind == 1) ready = deps_met(u) ? 1 : 0;
    }
    s_ready[b] = ready;
  };

  if (threadIdx.x == 0) {
    fetch(0);
    if (s_pos[0] < total && !s_ready[0]) {
      int kind, u, t;
      fused_decode<N>(s_pos[0], U, kind, u, t);
      wait_deps(u);
      s_ready[0] = 1;
    }
  }
  __syncthreads();  // twiddles, first position
  long pos = s_pos[0];
  if (pos >= total) return;
  float2 va[8], vb[8];
  {
    int kind, u, t;
    fused_decode<N>(pos, U, kind, u, t);
    load(va, kind, u, t);
  }
  int buf = 0;
  for (;;) {
    int kind, u, t;
    fused_decode<N>(pos, U, kind, u, t);
    // take the next position; its loads go out now if they need no wait
    if (threadIdx.x == 0) fetch(buf ^ 1);
    __syncthreads();
    const long npos = s_pos[buf ^ 1];
    const bool has_next = npos < total;
    bool next_loaded = false;
    int nkind = 0, nu = 0, nt = 0;
    if (has_next) {
      fused_decode<N>(npos, U, nkind, nu, nt);
      if (s_ready[buf ^ 1]) {
        load(vb, nkind, nu, nt);
        next_loaded = true;
      }
    }
    if (FftPP<N>::CALL_SYNC) __syncthreads();
    fft_line_pp<N, true>(va, s0, s1, stw, j);
    float2* p = tile_ptr(kind, u, t);
    if (kind == 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) p[(j + r * (N / 8)) * CW] = va[r];
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(ky_done + u, 1);
    } else {
      // the tile's N lines of CW values have been read by every thread (the
      // transform's exchanges are behind barriers): drop them from L2
      if (threadIdx.x < N) discard_l2_line(p - col + (long)threadIdx.x * astride);
      const int k = u / NBLK, cb = u % NBLK;
      const uint32_t ridx = (uint32_t)bt.r[k].ridx;
      const int c = cb * CW + col;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (is_centre(va[r], alpha, zmul)) {
          const long idx = ((long)(j + r * (N / 8)) * N + t) * N + c;
          const uint8_t old = __ldcg(rc + idx);
          if (ridx < old) rc[idx] = (uint8_t)ridx;
        }
      }
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(kx_done + u, 1);
    }
    if (!has_next) break;
    if (!next_loaded) {
      if (threadIdx.x == 0) wait_deps(nu);
      __syncthreads();
      load(vb, nkind, nu, nt);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) va[r] = vb[r];
    pos = npos;
    buf ^= 1;
  }
}

template <int N>
struct FusedLaunch {
  static cudaError_t setup() {
    return cudaFuncSetAttribute(k_cols_ba_fused<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)KGeom<N>::SMEM);
  }
  static cudaError_t launch(const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw, int* ctl, int* err,
                            int nsm, uint32_t lim, cudaStream_t st) {
    using X = KGeom<N>;
    const size_t ctl_bytes = sizeof(int) * (1 + 2 * (size_t)bt.K * CbGeom<N>::NBLK);
    cudaError_t e = cudaMemsetAsync(ctl, 0, ctl_bytes, st);
    if (e != cudaSuccess) return e;
    k_cols_ba_fused<N><<<nsm, X::THREADS, X::SMEM, st>>>(bt, rc, alpha, tw, ctl, err, lim);
    return cudaGetLastError();
  }
};

bool fused_supported(int N) { return N >= 64 && N <= 512; }

// ints of the control block for batches of up to KMAX radii
size_t fused_ctl_ints(int N) { return 1 + 2 * (size_t)KMAX * (N / CbGeom<512>::CW); }

cudaError_t fused_setup(int N) {
  switch (N) {
    case 64: return FusedLaunch<64>::setup();
    case 128: return FusedLaunch<128>::setup();
    case 256: return FusedLaunch<256>::setup();
    case 512: return FusedLaunch<512>::setup();
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_cols_ba_fused(int N, const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw, int* ctl,
                                 int* err, int nsm, cudaStream_t st, uint32_t spin_limit) {
  const uint32_t lim = spin_limit ? spin_limit : SF21_FUSED_SPIN_LIMIT;
  switch (N) {
    case 64: return FusedLaunch<64>::launch(bt, rc, alpha, tw, ctl, err, nsm, lim, st);
    case 128: return FusedLaunch<128>::launch(bt, rc, alpha, tw, ctl, err, nsm, lim, st);
    case 256: return FusedLaunch<256>::launch(bt, rc, alpha, tw, ctl, err, nsm, lim, st);
    case 512: return FusedLaunch<512>::launch(bt, rc, alpha, tw, ctl, err, nsm, lim, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sf21
