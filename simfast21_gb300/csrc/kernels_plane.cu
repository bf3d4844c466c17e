// Plane pass of the inverse transform: k-space top-hat filter + kz and ky
// transforms of a whole kx plane in one kernel, on a thread-block cluster.
//
// One cluster of C = N/32 CTAs owns the plane a (N x N complex): CTA `rank`
// holds rows b in [32 rank, 32 rank + 32) in shared memory.  Per radius:
//   1. each CTA filters and kz-transforms its 32 rows (rows read from HBM,
//      or from L2 for the second and later radii of the batch);
//   2. cluster barrier;
//   3. each CTA gathers its 32 columns c in [32 rank, 32 rank + 32) from the
//      32-row slices of all CTAs through distributed shared memory, ky-
//      transforms them and writes them to the radius' work box;
//   4. cluster barrier (the slices are rewritten by the next radius).
// The kz+ky intermediate never goes to HBM: per radius the plane pass costs
// one write of the work box (8 B/voxel) and the kx pass one read -- the
// 16 B/voxel radius round trip -- plus one spectrum read per batch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace cg = cooperative_groups;

namespace sf21 {

template <int N>
struct PlaneGeom {
  static constexpr int RPC = 32;                  // rows (and columns) per CTA
  static constexpr int C = N / RPC;               // CTAs per cluster
  static constexpr int T = N / 8;                 // threads per line
  static constexpr int THREADS = (RPC * T < 1024) ? RPC * T : 1024;
  static constexpr int LPG = THREADS / T;         // lines per group
  static constexpr int GROUPS = RPC / LPG;
  static constexpr int LS = LineGeom<N>::LS;
  static constexpr size_t SMEM = (size_t)(N + RPC * LS + LPG * LS) * sizeof(float2);
};

template <int N>
__global__ void __launch_bounds__(PlaneGeom<N>::THREADS, 1)
k_plane_filter(const float2* __restrict__ spec, Batch bt, const float2* __restrict__ gtw) {
  using G = PlaneGeom<N>;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* slice = dsm + N;
  float2* xch = slice + G::RPC * G::LS;
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
  const int rank = (int)cluster.block_rank();
  const int a = blockIdx.x / G::C;
  const int ka = kfreq(a, N);
  __syncthreads();
  for (int k = 0; k < bt.K; ++k) {
    const float dkR = bt.r[k].dkR;
    // 1. filter + kz transform of this CTA's rows (lanes along c)
    {
      const int line = threadIdx.x / G::T;
      const int j = threadIdx.x % G::T;
#pragma unroll 1
      for (int g = 0; g < G::GROUPS; ++g) {
        const int bl = g * G::LPG + line;
        const int b = rank * G::RPC + bl;
        const int kb = kfreq(b, N);
        const int kab = ka * ka + kb * kb;
        const float2* src = spec + ((long)a * N + b) * N;
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const int c = j + r * (N / 8);
          const int kc = kfreq(c, N);
          const float w = w_tophat(dkR * sqrtf((float)(kab + kc * kc)));
          const float2 zz = src[c];
          v[r] = filter_mul(zz, w);
        }
        float2* s = slice + bl * G::LS;
        fft_line<N, true>(v, s, stw, j);
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 8; ++r) s[padx(j + r * (N / 8))] = v[r];
      }
    }
    cluster.sync();
    // 3. ky transform of this CTA's columns (lanes along c)
    {
      const int cl_in = threadIdx.x % G::LPG;
      const int j = threadIdx.x / G::LPG;
      float2* dst = bt.r[k].work + (long)a * N * N;
#pragma unroll 1
      for (int g = 0; g < G::GROUPS; ++g) {
        const int cl = g * G::LPG + cl_in;
        const int c = rank * G::RPC + cl;
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const int b = j + r * (N / 8);
          const float2* rs = cluster.map_shared_rank(slice, b / G::RPC);
          v[r] = rs[(b % G::RPC) * G::LS + padx(c)];
        }
        fft_line<N, true>(v, xch + cl_in * G::LS, stw, j);
#pragma unroll
        for (int r = 0; r < 8; ++r) dst[(long)(j + r * (N / 8)) * N + c] = v[r];
      }
    }
    cluster.sync();
  }
}

template <int N>
static cudaError_t plane_setup_impl() {
  using G = PlaneGeom<N>;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_plane_filter<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM)))
    return e;
  if (G::C > 8) {
    if ((e = cudaFuncSetAttribute(k_plane_filter<N>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)))
      return e;
  }
  return cudaSuccess;
}

template <int N>
static cudaError_t plane_launch_impl(const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st) {
  using G = PlaneGeom<N>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(N * G::C), 1, 1);
  cfg.blockDim = dim3(G::THREADS, 1, 1);
  cfg.dynamicSmemBytes = G::SMEM;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G::C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_plane_filter<N>, spec, bt, tw);
}

template <int N>
static int plane_clusters_impl() {
  using G = PlaneGeom<N>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(N * G::C), 1, 1);
  cfg.blockDim = dim3(G::THREADS, 1, 1);
  cfg.dynamicSmemBytes = G::SMEM;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = G::C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_plane_filter<N>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

bool plane_supported(int N) { return N >= 64 && N <= 512; }

cudaError_t plane_setup(int N) {
  switch (N) {
    case 64: return plane_setup_impl<64>();
    case 128: return plane_setup_impl<128>();
    case 256: return plane_setup_impl<256>();
    case 512: return plane_setup_impl<512>();
    default: return cudaErrorInvalidValue;
  }
}

int plane_max_active_clusters(int N) {
  switch (N) {
    case 64: return plane_clusters_impl<64>();
    case 128: return plane_clusters_impl<128>();
    case 256: return plane_clusters_impl<256>();
    case 512: return plane_clusters_impl<512>();
    default: return 0;
  }
}

cudaError_t launch_plane_filter(int N, const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st) {
  switch (N) {
    case 64: return plane_launch_impl<64>(spec, bt, tw, st);
    case 128: return plane_launch_impl<128>(spec, bt, tw, st);
    case 256: return plane_launch_impl<256>(spec, bt, tw, st);
    case 512: return plane_launch_impl<512>(spec, bt, tw, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sf21
