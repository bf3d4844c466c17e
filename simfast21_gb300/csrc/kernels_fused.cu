// b- and a-axis inverse passes of a batch in one persistent launch, the
// b-axis output handed to the a-axis pass through L2 (radius pipeline 8).
//
// In the column-block-major work layout (kernels_cb.cu) the b- and a-axis
// transforms of one radius touch one column block's slab of N^2 CW values
// (32 MB at N = 512) and nothing else.  The launch walks the slabs ("units",
// u = k NBLK + cb for radius k of the batch and column block cb) in order:
// the b-axis tiles of a unit (fixed a: one contiguous N CW run, transformed
// in place) and, a little more than one unit later in the same queue, its
// a-axis tiles (fixed b: N runs of CW values N CW apart; transform, centre
// test, first-hit update).  So two to three slabs are live at a time, which
// L2 holds: the a-axis pass reads the b-axis output from L2 (ld.global.cg),
// and once a tile's lines have been read they are dropped from L2 without a
// write-back (discard.global.L2: the values are dead).  Per voxel and radius
// the DRAM sees the c-axis pass's write and the b-axis pass's read -- one
// HBM round trip per radius -- instead of two (ncu, K = 8:
// this launch reads the K boxes once and writes almost nothing, at 256^3 and
// at 512^3).
//
// Work queue: one CTA per SM takes queue items (groups of tiles, below) from
// an atomic counter.  An a-axis group of unit u waits until all N b-axis
// tiles of u have published (per-unit counter; the CTA's stores are ordered
// by a barrier, then one thread releases them with threadfence + atomic;
// acquire loads on the other side), and until the a-axis tiles of unit
// u - NBLK (the same column block at the previous radius) have finished (the
// radius order of the first-hit updates; these are atomicMin reductions into
// a 32-bit first-hit box, folded into bytes once per parameter set, so no
// warp waits on them).  b-axis groups never wait; a CTA waits only for its
// next item, after finishing its current one and publishing it, and what it
// waits for sits earlier in the queue, so the launch always completes.  The
// loads of the next tile -- of the same group, or the first of the next item
// when it needs no wait -- are issued before the current tile is transformed,
// and thread 0 takes queue positions two items ahead, so the latency of the
// queue atomics and of the dependency loads hides behind the transforms.
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

// Queue items are groups of G consecutive tiles of one kind and one unit
// (NG = N / G groups per unit and kind).  The item order merges the stream
// of b-axis groups (unit-major) with the stream of a-axis groups delayed by
// `lag` steps: step s takes b-axis group s, then a-axis group s - lag.  With
// lag = NG + slack, every a-axis group comes at least `slack` steps after the
// last b-axis group of its unit, so in the steady state its dependencies are
// already met when it is taken.
template <int N>
struct FusedGeom {
  static constexpr int G = 4;       // tiles per queue item (even: processed in pairs)
  static constexpr int NG = N / G;  // groups per unit and kind
};

__device__ __forceinline__ void fused_decode(int p, int Gy, int lag, int& kind, int& idx) {
  const int pairs_end = lag + 2 * (Gy - lag);
  if (p < lag) {
    kind = 0;
    idx = p;
  } else if (p < pairs_end) {
    const int q = p - lag;
    kind = q & 1;
    idx = kind ? q / 2 : lag + q / 2;
  } else {
    kind = 1;
    idx = p - Gy;
  }
}

template <int N>
__global__ void __launch_bounds__(KGeom<N>::THREADS, 1)
k_cols_ba_fused(Batch bt, unsigned int* __restrict__ rc32, const float* __restrict__ alpha_ptr,
                const float2* __restrict__ gtw, int* ctl, int* __restrict__ err, uint32_t spin_limit, int slack) {
  using Gm = CbGeom<N>;
  using X = KGeom<N>;
  using F = FusedGeom<N>;
  constexpr int CW = Gm::CW;
  constexpr int NBLK = Gm::NBLK;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  __shared__ int s_pos[3];    // queue positions of the next two items (ring of three slots)
  __shared__ int s_ready[3];  // 1: the item's loads may go out without a wait
  __shared__ int s_pend;      // counter index of the unpublished group, -1 none (thread 0)
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const float alpha = *alpha_ptr;
  const float zmul = bt.zmul;
  const int U = bt.K * NBLK;
  const int Gy = U * F::NG;  // b-axis groups (= a-axis groups)
  const int lag = min(Gy, F::NG + slack);
  const int total = 2 * Gy;
  int* head = ctl;
  int* ky_done = ctl + 1;
  int* kx_done = ctl + 1 + U;
  const int col = threadIdx.x % X::KW;
  const int j = threadIdx.x / X::KW;
  const long astride = (long)N * CW;
  float2* s0 = sbuf + col * X::LS;
  float2* s1 = sbuf + (X::KW + col) * X::LS;

  // dependencies of the a-axis groups of unit u (thread 0)
  auto deps_met = [&](int u) {
    if (ld_acquire_gpu(ky_done + u) < N) return false;
    return u < NBLK || ld_acquire_gpu(kx_done + u - NBLK) >= N;
  };
  auto wait_deps = [&](int u) {
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
  auto item = [&](int p, int& kind, int& u, int& t0) {
    int idx;
    fused_decode(p, Gy, lag, kind, idx);
    u = idx / F::NG;
    t0 = (idx % F::NG) * F::G;
  };
  // thread 0: readiness of the item at position p (b-axis items are always ready)
  auto ready_of = [&](int p) {
    if (p >= total) return 1;
    int kind, u, t0;
    item(p, kind, u, t0);
    return (kind == 0 || deps_met(u)) ? 1 : 0;
  };
  // completion of a group is published after the next group's first
  // transform, when its stores have drained, so the fence that orders them
  // is cheap; it is published at once before any wait (the awaited item may
  // depend on it)
  auto publish = [&]() {  // thread 0
    if (s_pend >= 0) {
      __threadfence();
      atomicAdd(ctl + s_pend, F::G);
      s_pend = -1;
    }
  };

  if (threadIdx.x == 0) {
    s_pend = -1;
    const int p0 = atomicAdd(head, 1);
    const int p1 = atomicAdd(head, 1);
    s_pos[0] = p0;
    s_pos[1] = p1;
    if (p0 < total && !ready_of(p0)) {
      int kind, u, t0;
      item(p0, kind, u, t0);
      wait_deps(u);
    }
    s_ready[1] = ready_of(p1);
  }
  __syncthreads();  // twiddles, first two positions
  const int pos = s_pos[0];
  if (pos >= total) return;
  int kind, u, t0;
  item(pos, kind, u, t0);
  float2 va[8], vb[8];
  load(va, kind, u, t0);
  int slot = 0;  // slot of the current item; (slot + 1) % 3 next, (slot + 2) % 3 the one after
  for (;;) {
    const int snext = slot == 2 ? 0 : slot + 1;
    const int safter = snext == 2 ? 0 : snext + 1;
    const int npos = s_pos[snext];
    const bool has_next = npos < total;
    const bool next_ready = has_next && s_ready[snext];
    int nkind = 0, nu = 0, nt0 = 0;
    if (has_next) item(npos, nkind, nu, nt0);
    // thread 0 takes the position after next now; it is used after the
    // group's first transform and published by the group-end barrier
    int pafter = total;
    if (threadIdx.x == 0 && has_next) pafter = atomicAdd(head, 1);
    bool next_loaded = false;
    const int k = u / NBLK, cb = u % NBLK;
    const unsigned int ridx = (unsigned int)bt.r[k].ridx;
    // transform + store (b axis) or centre test (a axis) of tile t held in v
    auto process = [&](float2 (&v)[8], int t, bool first) {
      if (FftPP<N>::CALL_SYNC) __syncthreads();
      fft_line_pp<N, true>(v, s0, s1, stw, j);
      if (first && threadIdx.x == 0) {
        publish();  // the previous group (every thread's stores precede the transform's barriers)
        if (has_next) {
          s_pos[safter] = pafter;
          s_ready[safter] = ready_of(pafter);  // acquire loads overlap the rest of the group
        }
      }
      float2* p = tile_ptr(kind, u, t);
      if (kind == 0) {
#pragma unroll
        for (int r = 0; r < 8; ++r) p[(j + r * (N / 8)) * CW] = v[r];
      } else {
        // every thread has read the tile's N lines of CW values (the
        // transform's exchanges are behind barriers): drop them from L2
        if (threadIdx.x < N) discard_l2_line(p - col + (long)threadIdx.x * astride);
        // first hit: a reduction nothing waits for
        const int c = cb * CW + col;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          if (is_centre(v[r], alpha, zmul)) atomicMin(rc32 + ((long)(j + r * (N / 8)) * N + t) * N + c, ridx);
        }
      }
    };
    // the group's tiles in pairs, the two register sets in turn (no copies):
    // each set's next tile -- or the next item's first tile -- is loaded
    // before the other set's transform
#pragma unroll 1
    for (int g = 0; g < F::G; g += 2) {
      load(vb, kind, u, t0 + g + 1);
      process(va, t0 + g, g == 0);
      if (g + 2 < F::G) {
        load(va, kind, u, t0 + g + 2);
      } else if (next_ready) {
        load(va, nkind, nu, nt0);
        next_loaded = true;
      }
      process(vb, t0 + g + 1, false);
    }
    // group done: every thread's stores are in; the release goes out later
    __syncthreads();
    if (threadIdx.x == 0) s_pend = (kind == 0 ? 1 : 1 + U) + u;
    if (!has_next) break;
    if (!next_loaded) {
      if (threadIdx.x == 0) {
        publish();
        wait_deps(nu);
      }
      __syncthreads();
      load(va, nkind, nu, nt0);
    }
    kind = nkind;
    u = nu;
    t0 = nt0;
    slot = snext;
  }
  if (threadIdx.x == 0) publish();
}

// The 32-bit first-hit box folded into the byte box the dilation reads
// (all bits set: never a centre).
__global__ void k_rc32_to_rc(long n3, const unsigned int* __restrict__ rc32, uint8_t* __restrict__ rc) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const unsigned int v = rc32[i];
    rc[i] = v < RC_NONE ? (uint8_t)v : RC_NONE;
  }
}

template <int N>
struct FusedLaunch {
  static cudaError_t setup() {
    return cudaFuncSetAttribute(k_cols_ba_fused<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)KGeom<N>::SMEM);
  }
  static cudaError_t launch(const Batch& bt, unsigned int* rc32, const float* alpha, const float2* tw, int* ctl,
                            int* err, int nsm, uint32_t lim, cudaStream_t st) {
    using X = KGeom<N>;
    const size_t ctl_bytes = sizeof(int) * (1 + 2 * (size_t)bt.K * CbGeom<N>::NBLK);
    cudaError_t e = cudaMemsetAsync(ctl, 0, ctl_bytes, st);
    if (e != cudaSuccess) return e;
    // slack: half a wave of CTAs between a unit's last b-axis group and its first a-axis group
    k_cols_ba_fused<N><<<nsm, X::THREADS, X::SMEM, st>>>(bt, rc32, alpha, tw, ctl, err, lim, nsm / 2);
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

cudaError_t launch_rc32_to_rc(long n3, const unsigned int* rc32, uint8_t* rc, cudaStream_t st) {
  k_rc32_to_rc<<<152 * 8, 256, 0, st>>>(n3, rc32, rc);
  return cudaGetLastError();
}

cudaError_t launch_cols_ba_fused(int N, const Batch& bt, unsigned int* rc32, const float* alpha, const float2* tw,
                                 int* ctl, int* err, int nsm, cudaStream_t st, uint32_t spin_limit) {
  const uint32_t lim = spin_limit ? spin_limit : SF21_FUSED_SPIN_LIMIT;
  switch (N) {
    case 64: return FusedLaunch<64>::launch(bt, rc32, alpha, tw, ctl, err, nsm, lim, st);
    case 128: return FusedLaunch<128>::launch(bt, rc32, alpha, tw, ctl, err, nsm, lim, st);
    case 256: return FusedLaunch<256>::launch(bt, rc32, alpha, tw, ctl, err, nsm, lim, st);
    case 512: return FusedLaunch<512>::launch(bt, rc32, alpha, tw, ctl, err, nsm, lim, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sf21
