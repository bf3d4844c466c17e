// The continuous ionisation criterion C(x) = max_R ion_R(x) / rec_R(x) and
// its vector-Jacobian product (hand-written adjoint).
//
// ion_R = zeta * B_R ion1, rec_R = B_R rec0 with B_R = IFFT(W_R FFT(.)) the
// (unnormalised, real, symmetric) top-hat filter of radius R, rec0 the
// recombination-rate box (get_HIIbubbles.c:222) and ion1 the zeta-free
// ionisation-rate box (:273).  The maximum runs over the radii of the FFT
// branch (R >= 2 dx, :299): below that the sharp k-space top-hat rings and
// the filtered recombination rate passes through zero, where the ratio is
// ill-conditioned (the small-R branch, :402-458, tests single cells).  Radii
// with rec_R(x) <= 0 do not compete (the reference's test treats them as
// automatic centres, :340-347, so they carry no ratio).  The forward keeps the running max and its radius index A(x)
// (uint8): the index is the only checkpoint; the backward recomputes the
// filtered fields radius by radius.
//
// Backward, for a cotangent g = dL/dC:
//   at voxels with A(x) = R:  dC/d rec_R = -C/rec_R,  dC/d ion1_R = zeta/rec_R,
//                             dC/d zeta = C/zeta,
//   grad rec0 + i alpha^-1... packed: Acc = sum_R W_R FFT(q_R),
//   q_R = g (-C/rec_R) + i (1/alpha) g zeta/rec_R   (masked by A = R),
//   IFFT(Acc) = sum_R B_R (dL/d rec_R) + i/alpha sum_R B_R (dL/d ion1_R)
// since B_R is its own adjoint.  Per batch of K radii: the recompute passes
// (same kernels as the forward), the kx pass that turns fields into
// cotangents and transforms them forward again, the ky forward pass, and the
// kz pass that multiplies by W_R, sums the K radii in registers and adds
// them to Acc once.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

template <int N>
struct AdjGeom {
  static constexpr int CW = (N <= 512) ? 16 : 8;
  static constexpr int THREADS = CW * (N / 8);
  static constexpr int T = N / 8;
  static constexpr int ROWS = (256 / T) > 0 ? (256 / T) : 1;
  static constexpr int RTHREADS = T * ROWS;
};

template <int N>
__device__ __forceinline__ void adj_load_tw(float2* stw, const float2* __restrict__ gtw) {
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
}

// Forward: kx inverse pass + running max of the ratio and its radius index.
template <int N>
__global__ void __launch_bounds__(AdjGeom<N>::THREADS)
k_cols_a_crit(Batch bt, float* __restrict__ Cbuf, uint8_t* __restrict__ Abuf, const float* __restrict__ alpha_ptr,
              const float2* __restrict__ gtw) {
  using G = AdjGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  adj_load_tw<N>(stw, gtw);
  const float alpha = fabsf(*alpha_ptr);  // sign: the no-source mark
  // no source anywhere: ion_R is exactly zero (the imaginary half is cross-talk)
  const float zmul = *alpha_ptr > 0.0f ? bt.zmul : 0.0f;
  const int nblk = N / G::CW;
  const long base = (long)(blockIdx.x / nblk) * N + (blockIdx.x % nblk) * G::CW;
  const long stride = (long)N * N;
  const int col = threadIdx.x % G::CW;
  const int j = threadIdx.x / G::CW;
  float best[8];
  int arg[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    best[r] = -INFINITY;
    arg[r] = RC_NONE;
  }
  for (int k = 0; k < bt.K; ++k) {
    const float2* box = bt.r[k].work;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = box[base + (long)(j + r * (N / 8)) * stride + col];
    __syncthreads();
    fft_line<N, true>(v, sbuf + col * L::LS, stw, j);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float den = v[r].x * alpha;  // alpha * rec_R
      if (den > 0.0f) {
        const float ratio = __fdiv_rn(v[r].y * zmul, den);
        if (ratio > best[r]) {
          best[r] = ratio;
          arg[r] = bt.r[k].ridx;
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    if (arg[r] != RC_NONE) {
      const long idx = base + (long)(j + r * (N / 8)) * stride + col;
      if (best[r] > Cbuf[idx]) {
        Cbuf[idx] = best[r];
        Abuf[idx] = (uint8_t)arg[r];
      }
    }
  }
}

// Backward kx pass: fields -> masked cotangents -> forward kx transform, in
// place in the batch's work boxes; per-block partial sum of g C / zeta.
template <int N>
__global__ void __launch_bounds__(AdjGeom<N>::THREADS)
k_cols_a_adj(Batch bt, const float* __restrict__ g, const uint8_t* __restrict__ Abuf,
             const float* __restrict__ alpha_ptr, float* __restrict__ zpart, const float2* __restrict__ gtw) {
  using G = AdjGeom<N>;
  using L = LineGeom<N>;
  extern __shared__ float2 dsm[];
  float2* stw = dsm;
  float2* sbuf = dsm + N;
  __shared__ float red[32];
  adj_load_tw<N>(stw, gtw);
  const float alpha = fabsf(*alpha_ptr);  // sign: the no-source mark
  const float inv_alpha = 1.0f / alpha;  // exact: alpha is a power of two
  const int nblk = N / G::CW;
  const long base = (long)(blockIdx.x / nblk) * N + (blockIdx.x % nblk) * G::CW;
  const long stride = (long)N * N;
  const int col = threadIdx.x % G::CW;
  const int j = threadIdx.x / G::CW;
  float zacc = 0.0f;
  for (int k = 0; k < bt.K; ++k) {
    float2* box = bt.r[k].work;
    const int ridx = bt.r[k].ridx;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = box[base + (long)(j + r * (N / 8)) * stride + col];
    __syncthreads();
    fft_line<N, true>(v, sbuf + col * L::LS, stw, j);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const long idx = base + (long)(j + r * (N / 8)) * stride + col;
      float2 q = make_float2(0.0f, 0.0f);
      if (Abuf[idx] == ridx) {
        const float rec = v[r].x;             // rec_R (> 0 where A = R)
        const float h = v[r].y * inv_alpha;   // ion1_R
        const float C = __fdiv_rn(bt.zmul * h, rec);
        const float gg = g[idx];
        const float ginv = __fdiv_rn(gg, rec);
        q = make_float2(-ginv * C, ginv * bt.zmul * inv_alpha);
        zacc += gg * __fdiv_rn(C, bt.zmul);
      }
      v[r] = q;
    }
    __syncthreads();
    fft_line<N, false>(v, sbuf + col * L::LS, stw, j);
#pragma unroll
    for (int r = 0; r < 8; ++r) box[base + (long)(j + r * (N / 8)) * stride + col] = v[r];
  }
  // deterministic block partial (accumulated over the batches in stream order)
  for (int o = 16; o > 0; o >>= 1) zacc += __shfl_xor_sync(0xffffffffu, zacc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = zacc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    zpart[blockIdx.x] += s;
  }
}

// Backward kz pass: forward kz transform of the K cotangent boxes, times
// W_R, summed over the batch and added to the k-space accumulator.
template <int N>
__global__ void __launch_bounds__(AdjGeom<N>::RTHREADS)
k_rows_adj_acc(Batch bt, float2* __restrict__ acc, const float2* __restrict__ gtw) {
  using G = AdjGeom<N>;
  using L = LineGeom<N>;
  __shared__ float2 stw[N];
  __shared__ float2 sbuf[G::ROWS * L::LS];
  adj_load_tw<N>(stw, gtw);
  const int row_in_cta = threadIdx.x / G::T;
  const int j = threadIdx.x % G::T;
  const long row = (long)blockIdx.x * G::ROWS + row_in_cta;
  const int a = (int)(row / N), b = (int)(row % N);
  const int ka = kfreq(a, N), kb = kfreq(b, N);
  const int kab = ka * ka + kb * kb;
  float kmag[8];
  float2 sum[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int kc = kfreq(j + r * (N / 8), N);
    kmag[r] = sqrtf((float)(kab + kc * kc));
    sum[r] = make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  for (int k = 0; k < bt.K; ++k) {
    const float2* src = bt.r[k].work + row * N;
    float2 v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = src[j + r * (N / 8)];
    fft_line<N, false>(v, sbuf + row_in_cta * L::LS, stw, j);
    const float dkR = bt.r[k].dkR;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const float w = w_tophat(dkR * kmag[r]);
      sum[r].x = fmaf(w, v[r].x, sum[r].x);
      sum[r].y = fmaf(w, v[r].y, sum[r].y);
    }
  }
  float2* dst = acc + row * N;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    float2 o = dst[j + r * (N / 8)];
    dst[j + r * (N / 8)] = make_float2(o.x + sum[r].x, o.y + sum[r].y);
  }
}

// Gradients with respect to the inputs from the inverse-transformed
// accumulator G = grad_rec0 + i grad_ion1 / alpha:
//   d rec0 / d delta = rec0 * 4 r3 / ((1+delta) (1 + (od/r2)^r3))   (user_functions.c:58-65)
//   d ion1 / d src   = the source multipliers (dx^3 Qion or (dx_s/dx_h)^3)
__global__ void k_grad_finish(long n3, const float2* __restrict__ Gbox, const float* __restrict__ alpha_ptr,
                              const float* __restrict__ delta, const float* __restrict__ rec0, float r2,
                              float r3, float src_mul, float* __restrict__ gdelta, float* __restrict__ gsrc) {
  const float alpha = fabsf(*alpha_ptr);  // sign: the no-source mark
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const float2 G = Gbox[i];
    const float od = 1.0f + delta[i];
    const float rec2 = powf(od / r2, r3);
    const float drec = rec0[i] * 4.0f * r3 / (od * (1.0f + rec2));
    if (gdelta) gdelta[i] = G.x * drec;
    if (gsrc) gsrc[i] = G.y * alpha * src_mul;
  }
}

__global__ void k_fill_crit_init(long n3, float* __restrict__ C, uint8_t* __restrict__ A) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    C[i] = -INFINITY;
    A[i] = RC_NONE;
  }
}

__global__ void k_crit_finalize(long n3, float* __restrict__ C, const uint8_t* __restrict__ A) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x)
    if (A[i] == RC_NONE) C[i] = 0.0f;
}

// ---- any box side (the shared-memory transform family): the same per-element
// rules over natural-layout work boxes, after whole-box transforms --------
constexpr int kAdjElemBlocks = 152 * 8;  // fixed grid: deterministic zeta partials

// Forward: running max of the ratio over the batch's fully inverse-transformed
// boxes (the rule of k_cols_a_crit).
__global__ void k_crit_elem(long n3, Batch bt, float* __restrict__ Cbuf, uint8_t* __restrict__ Abuf,
                            const float* __restrict__ alpha_ptr) {
  const float alpha = fabsf(*alpha_ptr);
  const float zmul = *alpha_ptr > 0.0f ? bt.zmul : 0.0f;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    float best = -INFINITY;
    int arg = RC_NONE;
    for (int k = 0; k < bt.K; ++k) {
      const float2 v = bt.r[k].work[i];
      const float den = v.x * alpha;
      if (den > 0.0f) {
        const float ratio = __fdiv_rn(v.y * zmul, den);
        if (ratio > best) {
          best = ratio;
          arg = bt.r[k].ridx;
        }
      }
    }
    if (arg != RC_NONE && best > Cbuf[i]) {
      Cbuf[i] = best;
      Abuf[i] = (uint8_t)arg;
    }
  }
}

// Backward: fields -> masked cotangents in place (the rule of k_cols_a_adj),
// per-block partial sums of g C / zeta.
__global__ void k_adj_elem(long n3, Batch bt, const float* __restrict__ g, const uint8_t* __restrict__ Abuf,
                           const float* __restrict__ alpha_ptr, float* __restrict__ zpart) {
  __shared__ float red[32];
  const float alpha = fabsf(*alpha_ptr);
  const float inv_alpha = 1.0f / alpha;  // exact: alpha is a power of two
  float zacc = 0.0f;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const int a = Abuf[i];
    for (int k = 0; k < bt.K; ++k) {
      float2 q = make_float2(0.0f, 0.0f);
      if (a == bt.r[k].ridx) {
        const float2 v = bt.r[k].work[i];
        const float rec = v.x;
        const float h = v.y * inv_alpha;
        const float C = __fdiv_rn(bt.zmul * h, rec);
        const float gg = g[i];
        const float ginv = __fdiv_rn(gg, rec);
        q = make_float2(-ginv * C, ginv * bt.zmul * inv_alpha);
        zacc += gg * __fdiv_rn(C, bt.zmul);
      }
      bt.r[k].work[i] = q;
    }
  }
  for (int o = 16; o > 0; o >>= 1) zacc += __shfl_xor_sync(0xffffffffu, zacc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = zacc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    zpart[blockIdx.x] += s;
  }
}

// Backward: acc += sum_k W(dk R_k |k|) box_k over the batch's forward-
// transformed cotangent boxes (the accumulation of k_rows_adj_acc).
__global__ void k_acc_elem(int N, Batch bt, float2* __restrict__ acc) {
  const long n3 = (long)N * N * N;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % N), b = (int)((i / N) % N), a = (int)(i / ((long)N * N));
    const int ka = kfreq(a, N), kb = kfreq(b, N), kc = kfreq(c, N);
    const float kmag = sqrtf((float)(ka * ka + kb * kb + kc * kc));
    float2 sum = make_float2(0.0f, 0.0f);
    for (int k = 0; k < bt.K; ++k) {
      const float w = w_tophat(bt.r[k].dkR * kmag);
      const float2 v = bt.r[k].work[i];
      sum.x = fmaf(w, v.x, sum.x);
      sum.y = fmaf(w, v.y, sum.y);
    }
    const float2 o = acc[i];
    acc[i] = make_float2(o.x + sum.x, o.y + sum.y);
  }
}

int adj_elem_blocks() { return kAdjElemBlocks; }
cudaError_t launch_crit_elem(long n3, const Batch& bt, float* C, uint8_t* A, const float* alpha, cudaStream_t st) {
  k_crit_elem<<<kAdjElemBlocks, 256, 0, st>>>(n3, bt, C, A, alpha);
  return cudaGetLastError();
}
cudaError_t launch_adj_elem(long n3, const Batch& bt, const float* g, const uint8_t* A, const float* alpha,
                            float* zpart, cudaStream_t st) {
  k_adj_elem<<<kAdjElemBlocks, 256, 0, st>>>(n3, bt, g, A, alpha, zpart);
  return cudaGetLastError();
}
cudaError_t launch_acc_elem(int N, const Batch& bt, float2* acc, cudaStream_t st) {
  k_acc_elem<<<kAdjElemBlocks, 256, 0, st>>>(N, bt, acc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
template <int N>
struct AdjLaunch {
  using G = AdjGeom<N>;
  static size_t smem() { return (N + G::CW * LineGeom<N>::LS) * sizeof(float2); }
  static unsigned grid_cols() { return (unsigned)((long)N * (N / G::CW)); }
  static cudaError_t setup() {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_cols_a_crit<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem())))
      return e;
    return cudaFuncSetAttribute(k_cols_a_adj<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem());
  }
  static cudaError_t crit(const Batch& bt, float* C, uint8_t* A, const float* alpha, const float2* tw,
                          cudaStream_t st) {
    k_cols_a_crit<N><<<grid_cols(), G::THREADS, smem(), st>>>(bt, C, A, alpha, tw);
    return cudaGetLastError();
  }
  static cudaError_t adj(const Batch& bt, const float* g, const uint8_t* A, const float* alpha, float* zpart,
                         const float2* tw, cudaStream_t st) {
    k_cols_a_adj<N><<<grid_cols(), G::THREADS, smem(), st>>>(bt, g, A, alpha, zpart, tw);
    return cudaGetLastError();
  }
  static cudaError_t rows_acc(const Batch& bt, float2* acc, const float2* tw, cudaStream_t st) {
    k_rows_adj_acc<N><<<(unsigned)((long)N * N / G::ROWS), G::RTHREADS, 0, st>>>(bt, acc, tw);
    return cudaGetLastError();
  }
};

#define SF21_ADJ_DISPATCH(N, CALL)                      \
  switch (N) {                                          \
    case 16: { using AL = AdjLaunch<16>; return CALL; }  \
    case 32: { using AL = AdjLaunch<32>; return CALL; }  \
    case 64: { using AL = AdjLaunch<64>; return CALL; }  \
    case 128: { using AL = AdjLaunch<128>; return CALL; } \
    case 256: { using AL = AdjLaunch<256>; return CALL; } \
    case 512: { using AL = AdjLaunch<512>; return CALL; } \
    case 1024: { using AL = AdjLaunch<1024>; return CALL; } \
    default: return cudaErrorInvalidValue;              \
  }

cudaError_t adj_setup(int N) { SF21_ADJ_DISPATCH(N, AL::setup()); }
int adj_zpart_blocks(int N) {
  const int cw = (N <= 512) ? 16 : 8;
  return N * (N / cw);
}
cudaError_t launch_cols_a_crit(int N, const Batch& bt, float* C, uint8_t* A, const float* alpha, const float2* tw,
                               cudaStream_t st) {
  SF21_ADJ_DISPATCH(N, AL::crit(bt, C, A, alpha, tw, st));
}
cudaError_t launch_cols_a_adj(int N, const Batch& bt, const float* g, const uint8_t* A, const float* alpha,
                              float* zpart, const float2* tw, cudaStream_t st) {
  SF21_ADJ_DISPATCH(N, AL::adj(bt, g, A, alpha, zpart, tw, st));
}
cudaError_t launch_rows_adj_acc(int N, const Batch& bt, float2* acc, const float2* tw, cudaStream_t st) {
  SF21_ADJ_DISPATCH(N, AL::rows_acc(bt, acc, tw, st));
}

static unsigned ew_grid(long n) {
  long b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? b : 152 * 32);
}
cudaError_t launch_grad_finish(long n3, const float2* G, const float* alpha, const float* delta, const float* rec0,
                               float r2, float r3, float src_mul, float* gdelta, float* gsrc, cudaStream_t st) {
  k_grad_finish<<<ew_grid(n3), 256, 0, st>>>(n3, G, alpha, delta, rec0, r2, r3, src_mul, gdelta, gsrc);
  return cudaGetLastError();
}
cudaError_t launch_crit_init(long n3, float* C, uint8_t* A, cudaStream_t st) {
  k_fill_crit_init<<<ew_grid(n3), 256, 0, st>>>(n3, C, A);
  return cudaGetLastError();
}
cudaError_t launch_crit_finalize(long n3, float* C, const uint8_t* A, cudaStream_t st) {
  k_crit_finalize<<<ew_grid(n3), 256, 0, st>>>(n3, C, A);
  return cudaGetLastError();
}

}  // namespace sf21
