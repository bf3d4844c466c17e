// Dilation of the bubble centres and the per-set finish of the xHII box.
//
// A voxel y is ionised by the radius loops iff some centre x with first-hit
// radius R_c(x) lies within the discrete ball of that radius:
// n(x, y) <= nmax(R_c(x)), n = squared per-axis minimum-image lattice
// distance (the sphere window of get_HIIbubbles.c:366 and the painting of
// :440-448).  Balls of smaller radii nest, so only the first (largest) hit
// matters.  With v(x) = nmax(R_c(x)) (-1 for no centre) the test is
//   max_x [v(x) - n(x, y)] >= 0,
// separable into three 1D max-plus passes with the kernel -d^2 (a, then b,
// then c).  Values below zero can never come back to >= 0, so every pass
// clamps them to -1, and a tap at distance d can only matter if d^2 <= the
// largest input value of the line, which bounds the window per tile.
//
// Each thread computes a strip of 8 consecutive outputs of one line.  Going
// outwards one distance d at a time, the 8 inputs at +d (and at -d) of the
// strip slide by one element per step, so they are kept in registers as two
// 8-element chunks on each side and refilled 8 elements at a time; every
// (output, distance) pair then costs one max and one fused add-max
// (__viaddmax_s32).  Chunks are 8-aligned and N is a multiple of 8, so
// periodic wrap never splits one.
//
// Data layout of the two intermediates (int per voxel):
//   I1 (after the a pass): column-block major with nc = dt_cols(N) columns,
//     ((c/nc N + b) N + a) nc + c%nc,
//     so that an a-pass tile (fixed b, 32 columns) writes one contiguous run
//     and a b-pass tile (fixed a) reads runs of 128 bytes inside one slab;
//   I2 (after the b pass): natural a N^2 + b N + c, read as rows by the
//     c pass, which also reads the per-voxel inputs of the finish as rows.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_kernels.h"
#include "softdouble.h"

namespace sf21 {

constexpr int DT_COLS = 32;       // columns of a column tile (N if N < 32)
constexpr int DT_THREADS = 512;
constexpr int DT_ROWS = 4;        // rows of a row tile (c pass)

__device__ __forceinline__ int isqrt_floor(int v) {
  int w = (int)sqrtf((float)v);
  while ((w + 1) * (w + 1) <= v) ++w;
  while (w * w > v) --w;
  return w;
}

// Number of 8-distance blocks needed for the largest value vmax of a tile.
__device__ __forceinline__ int dt_blocks(int vmax, int N) {
  if (vmax <= 0) return 0;
  int w = isqrt_floor(vmax);
  if (w > N / 2) w = N / 2;
  return (w + 7) / 8;
}

// Strip of 8 outputs y0..y0+7 (y0 multiple of 8) of one periodic line of
// length N; ld8(p, dst) loads the 8 elements p..p+7 (p multiple of 8, taken
// mod N by the caller's accessor).
// periodic index of a chunk start (N a multiple of 8: chunks never split)
__device__ __forceinline__ int dt_wrap(int x, int N) {
  x %= N;
  return x < 0 ? x + N : x;
}

template <class LD8>
__device__ __forceinline__ void dt_strip(const LD8& ld8, int y0, int nblk, int N, int (&acc)[8]) {
  int A[8], B[8], C[8], D[8];
  ld8(y0, A);
  ld8(dt_wrap(y0 + 8, N), B);
  ld8(dt_wrap(y0 - 8, N), C);
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    acc[r] = A[r];
    D[r] = A[r];
  }
  for (int m = 0; m < nblk; ++m) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int d = 8 * m + 1 + e;
      const int nd = -d * d;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int iu = e + 1 + r;  // in[y0 + r + d] = [A B][iu]
        const int id = 7 - e + r;  // in[y0 + r - d] = [C D][id]
        const int up = iu < 8 ? A[iu] : B[iu - 8];
        const int dn = id < 8 ? C[id] : D[id - 8];
        acc[r] = __viaddmax_s32(max(up, dn), nd, acc[r]);
      }
    }
    if (m + 1 < nblk) {
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        A[r] = B[r];
        D[r] = C[r];
      }
      ld8(dt_wrap(y0 + 8 * m + 16, N), B);
      ld8(dt_wrap(y0 - 8 * m - 16, N), C);
    }
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) acc[r] = acc[r] < -1 ? -1 : acc[r];
}

// columns of a column tile: the largest of 32, 16, 8 that divides N (N if N < 32)
__host__ __device__ __forceinline__ int dt_cols(int N) {
  return N < DT_COLS ? N : (N % 32 == 0 ? 32 : (N % 16 == 0 ? 16 : 8));
}

// Column tile: N lines of the pass axis x nc columns in shared memory,
// s[pos * (nc + 1) + col]; one warp = the 32 columns of one strip.
struct ColTileLd {
  const int* s;
  int col, ld;
  __device__ __forceinline__ void operator()(int p, int (&dst)[8]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) dst[i] = s[(p + i) * ld + col];
  }
};

__device__ __forceinline__ int block_max(int v, int* red) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  int m = -1;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = max(m, red[w]);
  return m;
}

// Pass along a, from rc (natural layout, uint8 first-hit index) to I1.
// blockIdx.x = cb N + b.
__global__ void __launch_bounds__(DT_THREADS, 2)
k_dt_pa(int N, const uint8_t* __restrict__ rc, const int* __restrict__ nmax, int* __restrict__ out) {
  extern __shared__ int s[];
  __shared__ int red[DT_THREADS / 32];
  const int nc = dt_cols(N), ldc = nc + 1;
  const int cb = blockIdx.x / N, b = blockIdx.x % N;
  const long nn = (long)N * N;
  int tmax = -1;
  for (int t = threadIdx.x; t < N * nc; t += blockDim.x) {
    const int a = t / nc, cc = t % nc;
    const uint8_t h = rc[a * nn + (long)b * N + cb * nc + cc];
    const int v = (h == RC_NONE) ? -1 : __ldg(nmax + h);
    s[a * ldc + cc] = v;
    tmax = max(tmax, v);
  }
  const int vmax = block_max(tmax, red);
  const int nblk = dt_blocks(vmax, N);
  int* dst = out + ((long)cb * N + b) * N * nc;
  const int col = threadIdx.x % nc;
  ColTileLd ld{s, col, ldc};
  for (int y0 = (threadIdx.x / nc) * 8; y0 < N; y0 += (blockDim.x / nc) * 8) {
    int acc[8];
    if (vmax < 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) acc[r] = -1;
    } else {
      dt_strip(ld, y0, nblk, N, acc);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) dst[(y0 + r) * nc + col] = acc[r];
  }
}

// Pass along b, I1 -> I2 (natural layout).  blockIdx.x = cb N + a.
__global__ void __launch_bounds__(DT_THREADS, 2)
k_dt_pb(int N, const int* __restrict__ in, int* __restrict__ out) {
  extern __shared__ int s[];
  __shared__ int red[DT_THREADS / 32];
  const int nc = dt_cols(N), ldc = nc + 1;
  const int cb = blockIdx.x / N, a = blockIdx.x % N;
  const long slab = (long)cb * N * N * nc;
  int tmax = -1;
  for (int t = threadIdx.x; t < N * nc; t += blockDim.x) {
    const int b = t / nc, cc = t % nc;
    const int v = in[slab + ((long)b * N + a) * nc + cc];
    s[b * ldc + cc] = v;
    tmax = max(tmax, v);
  }
  const int vmax = block_max(tmax, red);
  const int nblk = dt_blocks(vmax, N);
  int* dst = out + (long)a * N * N + cb * nc;
  const int col = threadIdx.x % nc;
  ColTileLd ld{s, col, ldc};
  for (int y0 = (threadIdx.x / nc) * 8; y0 < N; y0 += (blockDim.x / nc) * 8) {
    int acc[8];
    if (vmax < 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) acc[r] = -1;
    } else {
      dt_strip(ld, y0, nblk, N, acc);
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) dst[(long)(y0 + r) * N + col] = acc[r];
  }
}

// Row tile accessor: 8 consecutive ints of one row (16-byte aligned).
struct RowLd {
  const int* row;
  __device__ __forceinline__ void operator()(int p, int (&dst)[8]) const {
    const int4 u = *reinterpret_cast<const int4*>(row + p);
    const int4 w = *reinterpret_cast<const int4*>(row + p + 4);
    dst[0] = u.x; dst[1] = u.y; dst[2] = u.z; dst[3] = u.w;
    dst[4] = w.x; dst[5] = w.y; dst[6] = w.z; dst[7] = w.w;
  }
};

// Pass along c fused with the finish of the xHII box: single-cell fill
// (:281-288), inside-a-bubble (:392, :448) and the cap by the residual
// neutral fraction (:469-471).  chain = source chain before zeta (double
// bits), om = (1 - fresid) rounded down and to nearest, per voxel.
// blockIdx.x = group of DT_ROWS rows (a, b).  VEC: xhii is 16-byte aligned.
template <bool VEC>
__global__ void __launch_bounds__(DT_THREADS, 2)
k_dt_pc_finish(int N, const int* __restrict__ in, sd_t zeta, const sd_t* __restrict__ chain,
               const float* __restrict__ rec0, const float2* __restrict__ om, float* __restrict__ xhii) {
  extern __shared__ int s[];  // [DT_ROWS][N]
  __shared__ int red[DT_THREADS / 32];
  const long row0 = (long)blockIdx.x * DT_ROWS;
  int tmax = -1;
  for (int t = threadIdx.x; t < DT_ROWS * N / 4; t += blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(in + row0 * N)[t];
    reinterpret_cast<int4*>(s)[t] = v;
    tmax = max(tmax, max(max(v.x, v.y), max(v.z, v.w)));
  }
  const int vmax = block_max(tmax, red);
  const int nblk = dt_blocks(vmax, N);
  const int spr = N / 8;  // strips per row
  for (int q = threadIdx.x; q < DT_ROWS * spr; q += blockDim.x) {
    const int rr = q / spr, y0 = (q % spr) * 8;
    int acc[8];
    if (vmax < 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) acc[r] = -1;
    } else {
      RowLd ld{s + rr * N};
      dt_strip(ld, y0, nblk, N, acc);
    }
    const long i0 = (row0 + rr) * N + y0;
    float f[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const long i = i0 + r;
      if (acc[r] >= 0) {
        f[r] = 1.0f;
      } else {
        // h = (float)(chain(src) * zeta); fill = 1, h / rec0 or 0
        const float h = sd_to_float(sd_mul(chain[i], zeta));
        const float d0 = rec0[i];
        if (h > 0.0f)
          f[r] = (d0 > 0.0f) ? ((h >= d0) ? 1.0f : __fdiv_rn(h, d0)) : 1.0f;
        else
          f[r] = 0.0f;
      }
      // cap: f > (double)(1 - fresid) <=> f > om_down; value (float)(1 - fresid)
      const float2 o = om[i];
      if (f[r] > o.x) f[r] = o.y;
    }
    if (VEC) {
      float4* dst = reinterpret_cast<float4*>(xhii + i0);
      dst[0] = make_float4(f[0], f[1], f[2], f[3]);
      dst[1] = make_float4(f[4], f[5], f[6], f[7]);
    } else {
#pragma unroll
      for (int r = 0; r < 8; ++r) xhii[i0 + r] = f[r];
    }
  }
}

// Per-voxel inputs of the finish that do not depend on the parameter set,
// once per redshift: the source chain before zeta (double bits) and
// 1 - fresid rounded down / to nearest.
__global__ void k_finish_prep(long n3, const float* __restrict__ src, const float* __restrict__ fres,
                              const PrologueArgs pa, sd_t* __restrict__ chain, float2* __restrict__ om) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    sd_t t = sd_from_float(src[i]);
    for (int m = 0; m < pa.n_src_mul; ++m) t = sd_mul(t, pa.src_mul[m]);
    chain[i] = t;
    const sd_t o = sd_sub(0x3FF0000000000000ULL, sd_from_float(fres[i]));
    const float rn = sd_to_float(o);
    // largest float <= o
    const float lo = sd_gt(sd_from_float(rn), o) ? nextafterf(rn, -INFINITY) : rn;
    om[i] = make_float2(lo, rn);
  }
}

cudaError_t dt_setup(int N) {
  cudaError_t e;
  const int col_tile = N * (dt_cols(N) + 1) * (int)sizeof(int);
  const int row_tile = DT_ROWS * N * (int)sizeof(int);
  if ((e = cudaFuncSetAttribute(k_dt_pa, cudaFuncAttributeMaxDynamicSharedMemorySize, col_tile))) return e;
  if ((e = cudaFuncSetAttribute(k_dt_pb, cudaFuncAttributeMaxDynamicSharedMemorySize, col_tile))) return e;
  if ((e = cudaFuncSetAttribute(k_dt_pc_finish<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, row_tile)))
    return e;
  return cudaFuncSetAttribute(k_dt_pc_finish<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, row_tile);
}

// whole warps (the block reduction shuffles over all 32 lanes of every warp;
// threads past the last strip only load and reduce)
static int dt_threads(int N) {
  int t = N * dt_cols(N) / 8;
  t = (t + 31) / 32 * 32;
  return t < DT_THREADS ? t : DT_THREADS;
}
static size_t dt_col_smem(int N) { return (size_t)N * (dt_cols(N) + 1) * sizeof(int); }
static unsigned dt_col_grid(int N) { return (unsigned)((long)(N / dt_cols(N)) * N); }

cudaError_t launch_dt_pa(int N, const uint8_t* rc, const int* nmax, int* i1, cudaStream_t st) {
  if (N < 16) return cudaErrorInvalidValue;
  k_dt_pa<<<dt_col_grid(N), dt_threads(N), dt_col_smem(N), st>>>(N, rc, nmax, i1);
  return cudaGetLastError();
}

cudaError_t launch_dt_pb(int N, const int* i1, int* i2, cudaStream_t st) {
  if (N < 16) return cudaErrorInvalidValue;
  k_dt_pb<<<dt_col_grid(N), dt_threads(N), dt_col_smem(N), st>>>(N, i1, i2);
  return cudaGetLastError();
}

cudaError_t launch_dt_pc_finish(int N, const int* i2, uint64_t zeta, const uint64_t* chain, const float* rec0,
                                const float2* om, float* xhii, cudaStream_t st) {
  int thr = (DT_ROWS * N / 8 + 31) / 32 * 32;  // whole warps, as dt_threads
  thr = thr < DT_THREADS ? thr : DT_THREADS;
  const unsigned grid = (unsigned)((long)N * N / DT_ROWS);
  const size_t smem = (size_t)DT_ROWS * N * sizeof(int);
  if (((uintptr_t)xhii & 15) == 0)
    k_dt_pc_finish<true><<<grid, thr, smem, st>>>(N, i2, zeta, chain, rec0, om, xhii);
  else
    k_dt_pc_finish<false><<<grid, thr, smem, st>>>(N, i2, zeta, chain, rec0, om, xhii);
  return cudaGetLastError();
}

cudaError_t launch_finish_prep(long n3, const float* src, const float* fres, const PrologueArgs& pa, uint64_t* chain,
                               float2* om, cudaStream_t st) {
  long b = (n3 + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  k_finish_prep<<<(unsigned)b, 256, 0, st>>>(n3, src, fres, pa, chain, om);
  return cudaGetLastError();
}

}  // namespace sf21
