// Persistent, TMA-pipelined strided passes of the inverse transform.
//
// The ky pass (stride N) and the kx pass (stride N^2) read a tile of N rows
// x CW contiguous columns per line FFT batch.  Here each CTA (one per SM)
// walks a list of tiles; thread 0 issues the tensor-memory-accelerator copy
// of tile i+1 (cp.async.bulk.tensor, boxes of up to 256 rows, completing on
// an mbarrier) into the other half of a double buffer while all threads run
// the FFT of tile i, so HBM latency is overlapped with the FFT arithmetic.
// Results go straight from registers to HBM (ky pass, in place) or into the
// centre test and the first-hit update (kx pass; the filtered fields never
// return to HBM).
//
// Every mbarrier wait is bounded: after spin_limit polls (a launch argument,
// SF21_SPIN_LIMIT by default; the context can lower it) the CTA gives up,
// records the error in *err, waits for its own copies in flight (bounded by
// SF21_SPIN_LIMIT, whatever spin_limit is, so that no copy can still be
// writing into the CTA's shared memory when it exits) and returns; the host
// reads *err and reports SF21_E_TIMEOUT.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

#define SF21_SPIN_LIMIT (1u << 26)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {  // never suspends
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// At the default limit each poll is a try_wait (the thread may sleep until
// the phase completes or a system time limit passes); a lowered limit polls
// with test_wait, which returns at once, so the limit counts polls, not
// sleeps.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  if (limit >= SF21_SPIN_LIMIT) {
    for (uint32_t it = 0; it < limit; ++it)
      if (mbar_try_wait(bar, parity)) return true;
  } else {
    for (uint32_t it = 0; it < limit; ++it)
      if (mbar_test_wait(bar, parity)) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z,
                                            int w) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}

template <int N>
struct PipeGeom {
  static constexpr int CW = (N <= 512) ? 16 : 8;   // complex columns per tile (CW*8 B rows)
  static constexpr int THREADS = CW * (N / 8);
  static constexpr int BOX = N < 256 ? N : 256;    // rows per TMA box
  static constexpr int NBOX = N / BOX;
  static constexpr int LS = LineGeom<N>::LS;
  static constexpr size_t STAGE = (size_t)N * CW * sizeof(float2);
  static constexpr size_t STAGE_AL = (STAGE + 1023) & ~(size_t)1023;
  // [stage 0][stage 1][exchange CW lines][twiddles N][2 mbarriers]
  static constexpr size_t XOFF = 2 * STAGE_AL;
  static constexpr size_t TOFF = XOFF + (size_t)CW * LS * sizeof(float2);
  static constexpr size_t BOFF = (TOFF + (size_t)N * sizeof(float2) + 15) & ~(size_t)15;
  static constexpr size_t SMEM = BOFF + 2 * sizeof(uint64_t) + 1024;  // + alignment slack
};

// MODE 0: ky inverse pass, in place, over the K work boxes of the batch.
// MODE 1: kx inverse pass + centre test + first-hit update (K boxes per tile).
// LAYOUT 0: work boxes in the natural layout (a N^2 + b N + c);
// LAYOUT 1: column-block major (((c / CW) N + a) N + b) CW + c mod CW
// (kernels_cb.cu): a ky tile is one contiguous run, a kx tile stays inside
// one N^2 CW slab.  rc is in the natural layout either way.
template <int N, int MODE, int LAYOUT>
__global__ void __launch_bounds__(PipeGeom<N>::THREADS, 1)
k_pipe(const __grid_constant__ CUtensorMap tmap, Batch bt, float2* __restrict__ work0, long box_stride,
       uint8_t* __restrict__ rc, const float* __restrict__ alpha_ptr, const float2* __restrict__ gtw,
       int* __restrict__ err, uint32_t spin_limit) {
  using G = PipeGeom<N>;
  extern __shared__ __align__(1024) unsigned char pipe_smem_raw[];
  unsigned char* base_ptr =
      (unsigned char*)(((uintptr_t)pipe_smem_raw + 1023) & ~(uintptr_t)1023);
  float2* stage0 = (float2*)base_ptr;
  float2* stage1 = (float2*)(base_ptr + G::STAGE_AL);
  float2* xch = (float2*)(base_ptr + G::XOFF);
  float2* stw = (float2*)(base_ptr + G::TOFF);
  uint64_t* full = (uint64_t*)(base_ptr + G::BOFF);

  const int tid = threadIdx.x;
  const int col = tid % G::CW;
  const int j = tid / G::CW;
  const int nblk = N / G::CW;
  const int K = bt.K;
  const long tiles = (MODE == 0) ? (long)K * N * nblk : (long)N * nblk;
  const int per_tile = (MODE == 0) ? 1 : K;  // loads per tile
  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...
  const long my_tiles = tiles > blockIdx.x ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const long nloads = my_tiles * per_tile;

  for (int t = tid; t < N; t += blockDim.x) stw[t] = gtw[t];
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // decode load index -> (box k, outer index, column block)
  auto decode = [&](long li, int& k, int& outer, int& cb) {
    const long ti = li / per_tile;
    const long tile = blockIdx.x + ti * gridDim.x;
    if (LAYOUT == 1) {  // consecutive tiles are adjacent in memory
      if (MODE == 0) {
        k = (int)(tile / ((long)N * nblk));
        const long rem = tile % ((long)N * nblk);
        cb = (int)(rem / N);
        outer = (int)(rem % N);
      } else {
        k = (int)(li % per_tile);
        cb = (int)(tile / N);
        outer = (int)(tile % N);
      }
    } else if (MODE == 0) {
      k = (int)(tile / ((long)N * nblk));
      const long rem = tile % ((long)N * nblk);
      outer = (int)(rem / nblk);
      cb = (int)(rem % nblk);
    } else {
      k = (int)(li % per_tile);
      outer = (int)(tile / nblk);
      cb = (int)(tile % nblk);
    }
  };
  auto issue = [&](long li) {
    int k, outer, cb;
    decode(li, k, outer, cb);
    float2* dst = (li & 1) ? stage1 : stage0;
    uint64_t* bar = &full[li & 1];
    mbar_expect_tx(bar, (uint32_t)G::STAGE);
    const int wk = (int)((bt.r[k].work - work0) / box_stride);
    for (int q = 0; q < G::NBOX; ++q) {
      if (LAYOUT == 1) {  // map dims (2 CW floats, b, a, column block + nblk * box)
        if (MODE == 0)
          tma_load_4d(dst + (size_t)q * G::BOX * G::CW, &tmap, bar, 0, q * G::BOX, outer, wk * nblk + cb);
        else
          tma_load_4d(dst + (size_t)q * G::BOX * G::CW, &tmap, bar, 0, outer, q * G::BOX, wk * nblk + cb);
      } else if (MODE == 0)  // rows b, fixed a = outer
        tma_load_4d(dst + (size_t)q * G::BOX * G::CW, &tmap, bar, 2 * cb * G::CW, q * G::BOX, outer, wk);
      else            // rows a, fixed b = outer
        tma_load_4d(dst + (size_t)q * G::BOX * G::CW, &tmap, bar, 2 * cb * G::CW, outer, q * G::BOX, wk);
    }
  };

  if (tid == 0 && nloads > 0) issue(0);
  const float alpha = (MODE == 1) ? *alpha_ptr : 1.0f;
  int hit[8];
  long failed_at = -1;
  for (long li = 0; li < nloads; ++li) {
    if (tid == 0 && li + 1 < nloads) {
      fence_proxy_async();
      issue(li + 1);
    }
    const bool ok = mbar_wait_bounded(&full[li & 1], (uint32_t)((li >> 1) & 1), spin_limit);
    if (__syncthreads_or(!ok)) {
      failed_at = li;
      break;
    }
    int k, outer, cb;
    decode(li, k, outer, cb);
    const float2* st = (li & 1) ? stage1 : stage0;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = st[(j + r * (N / 8)) * G::CW + col];
    __syncthreads();  // stage free for the copy issued next iteration
    fft_line<N, true>(v, xch + col * G::LS, stw, j);
    const int c = cb * G::CW + col;
    if (MODE == 0 && LAYOUT == 1) {
      float2* box = bt.r[k].work + ((long)cb * N + outer) * N * G::CW + col;
#pragma unroll
      for (int r = 0; r < 8; ++r) box[(j + r * (N / 8)) * G::CW] = v[r];
    } else if (MODE == 0) {
      float2* box = bt.r[k].work + (long)outer * N * N + c;
#pragma unroll
      for (int r = 0; r < 8; ++r) box[(long)(j + r * (N / 8)) * N] = v[r];
    } else {
      if (k == 0) {
#pragma unroll
        for (int r = 0; r < 8; ++r) hit[r] = RC_NONE;
      }
      const int ridx = bt.r[k].ridx;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (is_centre(v[r], alpha, bt.zmul) && ridx < hit[r]) hit[r] = ridx;
      }
      if (k == per_tile - 1) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          if (hit[r] != RC_NONE) {
            const long idx = (long)outer * N + c + (long)(j + r * (N / 8)) * N * N;
            const uint8_t old = rc[idx];
            if (hit[r] < old) rc[idx] = (uint8_t)hit[r];
          }
        }
      }
    }
  }
  if (failed_at >= 0 && tid == 0) {
    atomicExch(err, 1);
    // drain this CTA's copies that may still be in flight (loads failed_at and
    // failed_at + 1) before its shared memory is released; bounded again
    (void)mbar_wait_bounded(&full[failed_at & 1], (uint32_t)((failed_at >> 1) & 1), SF21_SPIN_LIMIT);
    if (failed_at + 1 < nloads)
      (void)mbar_wait_bounded(&full[(failed_at + 1) & 1], (uint32_t)(((failed_at + 1) >> 1) & 1),
                              SF21_SPIN_LIMIT);
  }
}

// ---- host side ---------------------------------------------------------------
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static PFN_encodeTiled encode_fn() {
  static PFN_encodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_encodeTiled)p;
  }
  return fn;
}

// Tensor map over K contiguous N^3 complex boxes viewed as float32:
// natural layout (2N, N, N, K), column-block-major layout
// (2 CW, N, N, K N / CW); box (2 CW, rows, 1, 1) for the ky pass (rows along
// b) or (2 CW, 1, rows, 1) for the kx pass (rows along a).
static cudaError_t make_map(CUtensorMap* m, int N, int K, void* base, int cw, int box_rows, bool rows_along_a,
                            int layout = 0) {
  PFN_encodeTiled enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  cuuint64_t dims[4] = {(cuuint64_t)2 * N, (cuuint64_t)N, (cuuint64_t)N, (cuuint64_t)K};
  cuuint64_t strides[3] = {(cuuint64_t)2 * N * 4, (cuuint64_t)2 * N * N * 4, (cuuint64_t)2 * N * N * N * 4};
  if (layout == 1) {
    dims[0] = (cuuint64_t)2 * cw;
    dims[3] = (cuuint64_t)K * (N / cw);
    strides[0] = (cuuint64_t)2 * cw * 4;
    strides[1] = (cuuint64_t)2 * cw * N * 4;
    strides[2] = (cuuint64_t)2 * cw * N * N * 4;
  }
  cuuint32_t box[4] = {(cuuint32_t)(2 * cw), rows_along_a ? 1u : (cuuint32_t)box_rows,
                       rows_along_a ? (cuuint32_t)box_rows : 1u, 1u};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int N>
struct PipeLaunch {
  using G = PipeGeom<N>;
  static cudaError_t setup() {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_pipe<N, 0, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM)))
      return e;
    if ((e = cudaFuncSetAttribute(k_pipe<N, 1, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM)))
      return e;
    if ((e = cudaFuncSetAttribute(k_pipe<N, 0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM)))
      return e;
    return cudaFuncSetAttribute(k_pipe<N, 1, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
  }
  static cudaError_t maps(PipeMaps* pm, int K, void* base) {
    cudaError_t e;
    if ((e = make_map(&pm->b_rows, N, K, base, G::CW, G::BOX, false))) return e;
    if ((e = make_map(&pm->a_rows, N, K, base, G::CW, G::BOX, true))) return e;
    if ((e = make_map(&pm->b_rows_cb, N, K, base, G::CW, G::BOX, false, 1))) return e;
    return make_map(&pm->a_rows_cb, N, K, base, G::CW, G::BOX, true, 1);
  }
  static cudaError_t launch(int mode, int layout, const PipeMaps& pm, const Batch& bt, float2* work0, uint8_t* rc,
                            const float* alpha, const float2* tw, int* err, int nsm, uint32_t lim,
                            cudaStream_t st) {
    const long box_stride = (long)N * N * N;
    if (mode == 0 && layout == 0)
      k_pipe<N, 0, 0><<<nsm, G::THREADS, G::SMEM, st>>>(pm.b_rows, bt, work0, box_stride, rc, alpha, tw, err, lim);
    else if (mode == 1 && layout == 0)
      k_pipe<N, 1, 0><<<nsm, G::THREADS, G::SMEM, st>>>(pm.a_rows, bt, work0, box_stride, rc, alpha, tw, err, lim);
    else if (mode == 0)
      k_pipe<N, 0, 1><<<nsm, G::THREADS, G::SMEM, st>>>(pm.b_rows_cb, bt, work0, box_stride, rc, alpha, tw, err, lim);
    else
      k_pipe<N, 1, 1><<<nsm, G::THREADS, G::SMEM, st>>>(pm.a_rows_cb, bt, work0, box_stride, rc, alpha, tw, err, lim);
    return cudaGetLastError();
  }
};

bool pipe_supported(int N) { return N >= 64 && N <= 1024; }

cudaError_t pipe_setup(int N) {
  switch (N) {
    case 64: return PipeLaunch<64>::setup();
    case 128: return PipeLaunch<128>::setup();
    case 256: return PipeLaunch<256>::setup();
    case 512: return PipeLaunch<512>::setup();
    case 1024: return PipeLaunch<1024>::setup();
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t pipe_make_maps(int N, PipeMaps* pm, int K, void* work_base) {
  switch (N) {
    case 64: return PipeLaunch<64>::maps(pm, K, work_base);
    case 128: return PipeLaunch<128>::maps(pm, K, work_base);
    case 256: return PipeLaunch<256>::maps(pm, K, work_base);
    case 512: return PipeLaunch<512>::maps(pm, K, work_base);
    case 1024: return PipeLaunch<1024>::maps(pm, K, work_base);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_pipe(int N, int mode, int layout, const PipeMaps& pm, const Batch& bt, float2* work0,
                        uint8_t* rc, const float* alpha, const float2* tw, int* err, int nsm, cudaStream_t st,
                        uint32_t spin_limit) {
  const uint32_t lim = spin_limit ? spin_limit : SF21_SPIN_LIMIT;
  switch (N) {
    case 64: return PipeLaunch<64>::launch(mode, layout, pm, bt, work0, rc, alpha, tw, err, nsm, lim, st);
    case 128: return PipeLaunch<128>::launch(mode, layout, pm, bt, work0, rc, alpha, tw, err, nsm, lim, st);
    case 256: return PipeLaunch<256>::launch(mode, layout, pm, bt, work0, rc, alpha, tw, err, nsm, lim, st);
    case 512: return PipeLaunch<512>::launch(mode, layout, pm, bt, work0, rc, alpha, tw, err, nsm, lim, st);
    case 1024: return PipeLaunch<1024>::launch(mode, layout, pm, bt, work0, rc, alpha, tw, err, nsm, lim, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sf21
