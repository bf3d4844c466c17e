// Register-resident strided passes for the side N = 600 (the reference's
// default N_smoothed): the b- and a-axis line transforms of the HII stage.
//
// The shared-memory Stockham lines of kernels_gen.cu take every one of the
// four radix stages of 600 = 5 5 3 8 through shared memory.  Here a line is
// split once, 600 = 24 x 25 (input n = n1 + 24 n2, output k = 25 k1 + k2):
//   step 1: thread n1 holds x[n1 + 24 n2], n2 = 0..24, and computes the
//           25-point DFT over n2 in registers (5 x 5), then multiplies by the
//           twiddle w600^(n1 k2);
//   one exchange through shared memory;
//   step 2: thread k2 holds the 24 values of its k2 and computes the 24-point
//           DFT over n1 in registers (8 x 3); output k1 goes to row 25 k1 + k2.
// A tile is CW = 8 adjacent columns of one line set (fixed outer index);
// thread (col, r) has col = t mod 8, r = t / 8 (r = n1 in step 1, k2 in step
// 2), so a warp reads and writes 4 rows x 8 columns (64-byte runs) and the
// exchange (padded to 200 float2 per k2) is free of bank conflicts.  Inverse
// transforms use the conjugate twiddles; all are unnormalised (FFTW's
// convention, get_HIIbubbles.c:110-183).
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {
namespace g600 {
constexpr int N = 600, N1 = 24, N2 = 25, CW = 8, ROWS = 28;
constexpr int THREADS = CW * ROWS;       // 224: step 1 uses rows 0..23, step 2 rows 0..24
constexpr int EXS = N1 * CW + CW;        // float2 per k2 slab of the exchange (padded)
constexpr size_t SMEM = (size_t)(N + N2 * EXS) * sizeof(float2);  // twiddles, exchange
}  // namespace g600

template <bool INV>
__device__ __forceinline__ float2 twc(const float2* tw, int t) {  // w600^t, conjugated for the inverse
  float2 w = tw[t];
  if (INV) w.y = -w.y;
  return w;
}

// -i b (forward) or +i b (inverse) added to a: a - i b / a + i b
template <bool INV>
__device__ __forceinline__ float2 add_mi(float2 a, float2 b) {
  return INV ? make_float2(a.x - b.y, a.y + b.x) : make_float2(a.x + b.y, a.y - b.x);
}
template <bool INV>
__device__ __forceinline__ float2 sub_mi(float2 a, float2 b) {
  return INV ? make_float2(a.x + b.y, a.y - b.x) : make_float2(a.x - b.y, a.y + b.x);
}

// 5-point DFT in place (w = exp(-/+ 2 pi i / 5)).
template <bool INV>
__device__ __forceinline__ void dft5(float2& x0, float2& x1, float2& x2, float2& x3, float2& x4) {
  const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
  const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
  const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
  const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
  const float2 t1 = cadd(x1, x4), t2 = cadd(x2, x3), t3 = csub(x1, x4), t4 = csub(x2, x3);
  const float2 y0 = cadd(x0, cadd(t1, t2));
  const float2 a1 = make_float2(fmaf(c2, t2.x, fmaf(c1, t1.x, x0.x)), fmaf(c2, t2.y, fmaf(c1, t1.y, x0.y)));
  const float2 a2 = make_float2(fmaf(c1, t2.x, fmaf(c2, t1.x, x0.x)), fmaf(c1, t2.y, fmaf(c2, t1.y, x0.y)));
  const float2 b1 = make_float2(fmaf(s2, t4.x, __fmul_rn(s1, t3.x)), fmaf(s2, t4.y, __fmul_rn(s1, t3.y)));
  const float2 b2 = make_float2(fmaf(-s1, t4.x, __fmul_rn(s2, t3.x)), fmaf(-s1, t4.y, __fmul_rn(s2, t3.y)));
  x0 = y0;
  x1 = add_mi<INV>(a1, b1);
  x4 = sub_mi<INV>(a1, b1);
  x2 = add_mi<INV>(a2, b2);
  x3 = sub_mi<INV>(a2, b2);
}

// 3-point DFT in place (w = exp(-/+ 2 pi i / 3)).
template <bool INV>
__device__ __forceinline__ void dft3(float2& x0, float2& x1, float2& x2) {
  const float h3 = 0.86602540378443864676f;  // sqrt(3) / 2
  const float2 t = cadd(x1, x2);
  const float2 a = make_float2(fmaf(-0.5f, t.x, x0.x), fmaf(-0.5f, t.y, x0.y));
  const float2 d = csub(x1, x2);
  const float2 b = make_float2(__fmul_rn(h3, d.x), __fmul_rn(h3, d.y));
  x0 = cadd(x0, t);
  x1 = add_mi<INV>(a, b);
  x2 = sub_mi<INV>(a, b);
}

// 25-point DFT of y[n2] (5 x 5: n2 = 5 m1 + m2, k2 = l1 + 5 l2); on return
// y[5 l1 + l2] holds the output k2 = l1 + 5 l2.
template <bool INV>
__device__ __forceinline__ void dft25(float2 (&y)[25], const float2* tw) {
#pragma unroll
  for (int m2 = 0; m2 < 5; ++m2) dft5<INV>(y[m2], y[5 + m2], y[10 + m2], y[15 + m2], y[20 + m2]);
#pragma unroll
  for (int l1 = 1; l1 < 5; ++l1)
#pragma unroll
    for (int m2 = 1; m2 < 5; ++m2) y[5 * l1 + m2] = cmul(y[5 * l1 + m2], twc<INV>(tw, 24 * m2 * l1));  // w25^(m2 l1)
#pragma unroll
  for (int l1 = 0; l1 < 5; ++l1) dft5<INV>(y[5 * l1], y[5 * l1 + 1], y[5 * l1 + 2], y[5 * l1 + 3], y[5 * l1 + 4]);
}

// 24-point DFT of u[n1] (8 x 3: n1 = 3 p1 + p2, k1 = q1 + 8 q2); on return
// u[3 q1 + q2] holds the output k1 = q1 + 8 q2.
template <bool INV>
__device__ __forceinline__ void dft24(float2 (&u)[24], const float2* tw) {
#pragma unroll
  for (int p2 = 0; p2 < 3; ++p2) {
    float2 v[8];
#pragma unroll
    for (int p1 = 0; p1 < 8; ++p1) v[p1] = u[3 * p1 + p2];
    dft8<INV>(v);
#pragma unroll
    for (int q1 = 0; q1 < 8; ++q1) u[3 * q1 + p2] = v[q1];
  }
#pragma unroll
  for (int q1 = 1; q1 < 8; ++q1)
#pragma unroll
    for (int p2 = 1; p2 < 3; ++p2) u[3 * q1 + p2] = cmul(u[3 * q1 + p2], twc<INV>(tw, 25 * p2 * q1));  // w24^(p2 q1)
#pragma unroll
  for (int q1 = 0; q1 < 8; ++q1) dft3<INV>(u[3 * q1], u[3 * q1 + 1], u[3 * q1 + 2]);
}

// EPI 0: transform in place (box0, or the batch's K boxes); EPI 1: inverse,
// centre test and first-hit update of the batch's K boxes (the transform is
// not stored).  AXIS 1: lines along b; AXIS 0: along a.  LAYOUT 0: natural
// boxes (a N^2 + b N + c: a-axis rows N^2 apart, 600 rows of a tile on 600
// pages); LAYOUT 1: the radius batch's work boxes column-block major,
// ((c / 8) N + a) N + b) 8 + c mod 8, where a b-axis tile is one contiguous
// run and an a-axis tile stays inside one 23 MB slab.
template <bool INV, int EPI, int AXIS, int LAYOUT>
__global__ void __launch_bounds__(g600::THREADS, 3) k_gen600_cols(float2* box0, Batch bt, uint8_t* rc,
                                                               const float* __restrict__ alpha_ptr,
                                                               const float2* __restrict__ gtw) {
  using namespace g600;
  extern __shared__ float2 gsm[];
  float2* tw = gsm;
  float2* ex = gsm + N;
  for (int t = threadIdx.x; t < N; t += THREADS) tw[t] = gtw[t];
  const int col = threadIdx.x % CW, r = threadIdx.x / CW;
  const int nblk = N / CW;
  const int outer = blockIdx.x / nblk;
  const int c0 = (blockIdx.x % nblk) * CW;
  constexpr long stride = LAYOUT == 1 ? (AXIS == 1 ? (long)CW : (long)N * CW) : (AXIS == 1 ? (long)N : (long)N * N);
  const long cbk = c0 / CW;
  const long base = LAYOUT == 1 ? (AXIS == 1 ? (cbk * N + outer) * N * CW : (cbk * N * N + outer) * CW) + col
                                : (AXIS == 1 ? (long)outer * N * N : (long)outer * N) + c0 + col;
  const int nbox = box0 ? 1 : bt.K;
  float alpha = 1.0f;
  if (EPI == 1) alpha = *alpha_ptr;
  // EPI 1: first hits of this thread's 24 outputs (rows 25 k1 + r), over the
  // batch's radii in increasing index order: bit e of hmask says output e has
  // one, its radius index is byte e of hbyte (24 bytes in 6 words)
  uint32_t hmask = 0u;
  uint32_t hbyte[6] = {0u, 0u, 0u, 0u, 0u, 0u};
  for (int k = 0; k < nbox; ++k) {
    float2* box = box0 ? box0 : bt.r[k].work;
    __syncthreads();  // twiddles (k = 0); the previous box's step 2 is done with the exchange
    if (r < N1) {
      float2 y[25];
      const float2* src = box + base + (long)r * stride;
#pragma unroll
      for (int n2 = 0; n2 < 25; ++n2) y[n2] = src[(long)N1 * n2 * stride];
      dft25<INV>(y, tw);
#pragma unroll
      for (int l1 = 0; l1 < 5; ++l1)
#pragma unroll
        for (int l2 = 0; l2 < 5; ++l2) {
          const int k2 = l1 + 5 * l2;
          float2 v = y[5 * l1 + l2];
          if (k2 > 0 && r > 0) v = cmul(v, twc<INV>(tw, r * k2));  // w600^(n1 k2)
          ex[k2 * EXS + r * CW + col] = v;
        }
    }
    __syncthreads();
    if (r < N2) {
      float2 u[24];
#pragma unroll
      for (int n1 = 0; n1 < 24; ++n1) u[n1] = ex[r * EXS + n1 * CW + col];
      dft24<INV>(u, tw);
      if (EPI == 0) {
        float2* dst = box + base + (long)r * stride;
#pragma unroll
        for (int q1 = 0; q1 < 8; ++q1)
#pragma unroll
          for (int q2 = 0; q2 < 3; ++q2) dst[(long)25 * (q1 + 8 * q2) * stride] = u[3 * q1 + q2];
      } else {
        const uint32_t ridx = (uint32_t)bt.r[k].ridx;
#pragma unroll
        for (int e = 0; e < 24; ++e) {
          if (is_centre(u[e], alpha, bt.zmul) && !((hmask >> e) & 1u)) {
            hmask |= 1u << e;
            hbyte[e >> 2] |= ridx << (8 * (e & 3));
          }
        }
      }
    }
  }
  if (EPI == 1 && r < N2 && hmask) {
    // rc is in the natural layout (AXIS 0: row = a, outer = b); output e =
    // 3 q1 + q2 is row 25 (q1 + 8 q2) + r
#pragma unroll
    for (int e = 0; e < 24; ++e) {
      if ((hmask >> e) & 1u) {
        const int row = 25 * (e / 3 + 8 * (e % 3)) + r;
        const uint8_t h = (uint8_t)(hbyte[e >> 2] >> (8 * (e & 3)));
        const long idx = ((long)row * N + outer) * N + c0 + col;
        if (h < rc[idx]) rc[idx] = h;
      }
    }
  }
}

bool gen600_supported(int N) { return N == g600::N; }

// ---- c-axis (rows) pass: one warp per row ---------------------------------
// Lane n1 < 24 holds x[n1 + 24 n2] (for fixed n2 the 24 lanes read 24
// consecutive values: coalesced); lane k2 < 25 holds the outputs 25 k1 + k2
// (for fixed k1, 25 consecutive values: coalesced stores).  The exchange is
// the warp's own shared-memory block (stride 25 float2 per k2: the reads by
// k2 meet distinct banks), so a row needs no CTA barrier.
// MODE 0: forward, imaginary part times |alpha| (the packed prologue box);
// MODE 1: inverse in place; MODE 2: inverse of the spectrum row times the
// top-hat filter of each of the batch's K radii, into the K work boxes.
// In MODE 2 the window takes one value per |k_c| (c and N - c share it): all
// 32 lanes evaluate the row's N/2 + 1 values once per radius into a
// shared-memory row, instead of 24 lanes evaluating 25 each.  Same
// expression, same bits.
namespace g600 {
constexpr int RW = 8;                      // rows (warps) per CTA
constexpr int RTHREADS = 32 * RW;
constexpr int XS = N2 * N2;                // exchange float2 per warp (25 k2 x stride 25)
constexpr int WS = (N / 2 + 2) / 2;        // window row per warp, in float2 (N/2 + 1 floats, padded)
constexpr int NW = (N / 2 + 32) / 32;      // window values per lane
// twiddles; per warp: exchange, spectrum row, window row
constexpr size_t RSMEM = (size_t)(N + RW * (XS + N + WS)) * sizeof(float2);
}  // namespace g600

template <int MODE, int LAYOUT>
__global__ void __launch_bounds__(g600::RTHREADS, 2) k_gen600_rows(const float2* in, float2* out, Batch bt,
                                                                  const float* __restrict__ alpha_ptr,
                                                                  const float2* __restrict__ gtw) {
  using namespace g600;
  constexpr bool INV = MODE != 0;
  extern __shared__ float2 gsm[];
  float2* tw = gsm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float2* ex = gsm + N + w * (XS + N + WS);
  float2* zrow = ex + XS;
  float* wrow = reinterpret_cast<float*>(zrow + N);
  for (int t = threadIdx.x; t < N; t += RTHREADS) tw[t] = gtw[t];
  __syncthreads();
  const long row = (long)blockIdx.x * RW + w;
  const float2* src = in + row * N;
  const int nout = MODE == 2 ? bt.K : 1;
  float alpha = 1.0f;
  if (MODE == 0 && alpha_ptr) alpha = fabsf(*alpha_ptr);
  float kmag[NW];  // MODE 2: |k| at |k_c| = lane + 32 i (<= N/2) of this row
  if (MODE == 2) {
    const int a = (int)(row / N), b = (int)(row % N);
    const int ka = kfreq(a, N), kb = kfreq(b, N);
    const int kab = ka * ka + kb * kb;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      const int kc = lane + 32 * i;
      kmag[i] = kc <= N / 2 ? sqrtf((float)(kab + kc * kc)) : 0.0f;
    }
    for (int c = lane; c < N; c += 32) zrow[c] = src[c];
  }
  for (int k = 0; k < nout; ++k) {
    if (MODE == 2) {  // the window of radius k at every |k_c|
      const float dkR = bt.r[k].dkR;
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        const int kc = lane + 32 * i;
        if (kc <= N / 2) wrow[kc] = w_tophat(dkR * kmag[i]);
      }
      __syncwarp();
    }
    if (lane < N1) {
      float2 y[25];
#pragma unroll
      for (int n2 = 0; n2 < 25; ++n2) {
        const int c = lane + N1 * n2;
        if (MODE == 2) {
          y[n2] = filter_mul(zrow[c], wrow[c <= N / 2 ? c : N - c]);
        } else {
          float2 v = src[c];
          if (MODE == 0) v.y *= alpha;
          y[n2] = v;
        }
      }
      dft25<INV>(y, tw);
#pragma unroll
      for (int l1 = 0; l1 < 5; ++l1)
#pragma unroll
        for (int l2 = 0; l2 < 5; ++l2) {
          const int k2 = l1 + 5 * l2;
          float2 v = y[5 * l1 + l2];
          if (k2 > 0 && lane > 0) v = cmul(v, twc<INV>(tw, lane * k2));  // w600^(n1 k2)
          ex[k2 * N2 + lane] = v;
        }
    }
    __syncwarp();
    if (lane < N2) {
      float2 u[24];
#pragma unroll
      for (int n1 = 0; n1 < 24; ++n1) u[n1] = ex[lane * N2 + n1];
      dft24<INV>(u, tw);
      if (LAYOUT == 0) {
        float2* dst = (MODE == 2 ? bt.r[k].work : out) + row * N + lane;
#pragma unroll
        for (int q1 = 0; q1 < 8; ++q1)
#pragma unroll
          for (int q2 = 0; q2 < 3; ++q2) dst[25 * (q1 + 8 * q2)] = u[3 * q1 + q2];
      } else {  // column-block major: (a, b, c) at ((c / 8) N^2 + a N + b) 8 + c mod 8, row = a N + b
        float2* dst = (MODE == 2 ? bt.r[k].work : out) + row * CW;
#pragma unroll
        for (int q1 = 0; q1 < 8; ++q1)
#pragma unroll
          for (int q2 = 0; q2 < 3; ++q2) {
            const int c = 25 * (q1 + 8 * q2) + lane;
            dst[(long)(c / CW) * N * N * CW + c % CW] = u[3 * q1 + q2];
          }
      }
    }
    __syncwarp();  // the exchange is free for the next radius
  }
}

template <bool INV, int EPI, int AXIS, int LAYOUT>
static cudaError_t g600_attr() {
  return cudaFuncSetAttribute(k_gen600_cols<INV, EPI, AXIS, LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)g600::SMEM);
}

cudaError_t gen600_setup() {
  cudaError_t e;
  if ((e = g600_attr<true, 0, 0, 0>()) || (e = g600_attr<true, 0, 1, 0>()) || (e = g600_attr<false, 0, 0, 0>()) ||
      (e = g600_attr<false, 0, 1, 0>()) || (e = g600_attr<true, 0, 1, 1>()) || (e = g600_attr<true, 1, 0, 1>()))
    return e;
  for (auto f : {k_gen600_rows<0, 0>, k_gen600_rows<1, 0>, k_gen600_rows<2, 0>, k_gen600_rows<2, 1>})
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g600::RSMEM))) return e;
  return cudaSuccess;
}

cudaError_t launch_gen600_rows(int mode, const float2* in, float2* out, const Batch& bt, const float* alpha,
                               const float2* tw, bool cb, cudaStream_t st) {
  const unsigned grid = (unsigned)((long)g600::N * g600::N / g600::RW);
  const int T = g600::RTHREADS;
  const size_t S = g600::RSMEM;
  if (mode == 0)
    k_gen600_rows<0, 0><<<grid, T, S, st>>>(in, out, bt, alpha, tw);
  else if (mode == 1)
    k_gen600_rows<1, 0><<<grid, T, S, st>>>(in, out, bt, nullptr, tw);
  else if (cb)
    k_gen600_rows<2, 1><<<grid, T, S, st>>>(in, nullptr, bt, nullptr, tw);
  else
    k_gen600_rows<2, 0><<<grid, T, S, st>>>(in, nullptr, bt, nullptr, tw);
  return cudaGetLastError();
}

cudaError_t launch_gen600_cols(float2* box0, const Batch& bt, int axis, bool inverse, bool cb, const float2* tw,
                               cudaStream_t st) {
  const unsigned grid = (unsigned)(g600::N * (g600::N / g600::CW));
  const int T = g600::THREADS;
  const size_t S = g600::SMEM;
  if (cb) {  // the radius batch's b-axis inverse
    if (box0 || axis != 1 || !inverse) return cudaErrorInvalidValue;
    k_gen600_cols<true, 0, 1, 1><<<grid, T, S, st>>>(nullptr, bt, nullptr, nullptr, tw);
  } else if (inverse && axis == 1) {
    k_gen600_cols<true, 0, 1, 0><<<grid, T, S, st>>>(box0, bt, nullptr, nullptr, tw);
  } else if (inverse) {
    k_gen600_cols<true, 0, 0, 0><<<grid, T, S, st>>>(box0, bt, nullptr, nullptr, tw);
  } else if (axis == 1) {
    k_gen600_cols<false, 0, 1, 0><<<grid, T, S, st>>>(box0, bt, nullptr, nullptr, tw);
  } else {
    k_gen600_cols<false, 0, 0, 0><<<grid, T, S, st>>>(box0, bt, nullptr, nullptr, tw);
  }
  return cudaGetLastError();
}

cudaError_t launch_gen600_cols_a_test(const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                                      cudaStream_t st) {
  const unsigned grid = (unsigned)(g600::N * (g600::N / g600::CW));
  k_gen600_cols<true, 1, 0, 1><<<grid, g600::THREADS, g600::SMEM, st>>>(nullptr, bt, rc, alpha, tw);
  return cudaGetLastError();
}

}  // namespace sf21
