// Transforms of any box side N = 2^a 3^b 5^c (8 | N, 24 <= N <= 1280): the
// reference's recommended sides ("products of small primes (2, 3, 5)",
// simfast21.ini), e.g. its defaults N_smoothed = 600 and N_halo = 1200, which
// the power-of-two register FFT (fft_line.cuh) does not cover.
//
// Line FFT: Stockham autosort in shared memory with radix-8/4/2/3/5 stages,
//   stage (radix R, span Ns = product of the earlier radices, M = N/R):
//     v[r] = x[j + r M] * w^(k r N/(Ns R)),  k = j mod Ns,  V = DFT_R(v),
//     y[(j / Ns) Ns R + k + r Ns] = V[r]
// with w = exp(-2 pi i / N) from a table rounded once from double; all
// threads of a CTA share the butterflies of the CTA's lines, one barrier per
// stage.  Transforms are unnormalised, forward sign -1, inverse +1 (FFTW's
// convention, as the power-of-two path).
//
// Passes over natural-layout boxes (index (a N + b) N + c):
//   rows (c axis): LPC lines per CTA, loaded and stored as contiguous rows;
//     forward (with the packed imaginary part scaled by alpha), or inverse
//     with the HII top-hat filter of K radii (get_HIIbubbles.c:305-322) or
//     the halo finder's pair filter (get_halos.c:211-225);
//   columns (b or a axis): a tile of CW contiguous columns x N rows, loaded
//     as CW-element runs into CW lines; the a-axis inverse ends in the HII
//     centre test + first-hit update or in the halo thresholds.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "sf21_device.cuh"
#include "sf21_kernels.h"

namespace sf21 {

// ---- radix kernels (in registers) ----
template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

// x1 = a + b w, x2 = a + b w^2 with w = exp(-/+ 2 pi i / 3)
template <bool INV>
__device__ __forceinline__ void dft3(float2& x0, float2& x1, float2& x2) {
  const float s = INV ? -0.86602540378443864676f : 0.86602540378443864676f;  // sin(2 pi / 3), sign of -i
  const float2 t1 = cadd(x1, x2), t2 = csub(x1, x2);
  const float2 m = make_float2(x0.x - 0.5f * t1.x, x0.y - 0.5f * t1.y);
  // -i s t2 = (s t2.y, -s t2.x)
  const float2 r = make_float2(s * t2.y, -s * t2.x);
  x0 = cadd(x0, t1);
  x1 = cadd(m, r);
  x2 = csub(m, r);
}

template <bool INV>
__device__ __forceinline__ void dft5(float2& x0, float2& x1, float2& x2, float2& x3, float2& x4) {
  const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;  // cos(2 pi/5), cos(4 pi/5)
  const float s1 = INV ? -0.95105651629515357212f : 0.95105651629515357212f;  // sin(2 pi/5)
  const float s2 = INV ? -0.58778525229247312917f : 0.58778525229247312917f;  // sin(4 pi/5)
  const float2 p1 = cadd(x1, x4), m1 = csub(x1, x4), p2 = cadd(x2, x3), m2 = csub(x2, x3);
  const float2 a1 = make_float2(x0.x + c1 * p1.x + c2 * p2.x, x0.y + c1 * p1.y + c2 * p2.y);
  const float2 a2 = make_float2(x0.x + c2 * p1.x + c1 * p2.x, x0.y + c2 * p1.y + c1 * p2.y);
  const float2 b1 = make_float2(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);
  const float2 b2 = make_float2(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y);
  x0 = cadd(x0, cadd(p1, p2));
  // y1 = a1 - i b1, y4 = a1 + i b1, y2 = a2 - i b2, y3 = a2 + i b2 (-i b = (b.y, -b.x))
  x1 = make_float2(a1.x + b1.y, a1.y - b1.x);
  x4 = make_float2(a1.x - b1.y, a1.y + b1.x);
  x2 = make_float2(a2.x + b2.y, a2.y - b2.x);
  x3 = make_float2(a2.x - b2.y, a2.y + b2.x);
}

template <bool INV>
__device__ __forceinline__ void gen_butterfly(int R, float2 (&v)[8]) {
  switch (R) {
    case 8: dft8<INV>(v); break;
    case 4: dft4<INV>(v[0], v[1], v[2], v[3]); break;
    case 5: dft5<INV>(v[0], v[1], v[2], v[3], v[4]); break;
    case 3: dft3<INV>(v[0], v[1], v[2]); break;
    default: dft2<INV>(v[0], v[1]); break;
  }
}

// L lines of N elements at x + l ld (l < L); scratch y likewise.  All CTA
// threads take part (callers must reach it with every thread).  Returns the
// buffer (x or y) that holds the result.
template <bool INV>
__device__ float2* gen_fft_lines(float2* x, float2* y, int L, int ld, const GenPlan& p, const float2* __restrict__ tw) {
  const int N = p.N;
  float2* in = x;
  float2* out = y;
  int Ns = 1;
  for (int st = 0; st < p.nst; ++st) {
    const int R = p.radix[st];
    const int M = N / R;
    const int tstep = N / (Ns * R);
    for (int g = threadIdx.x; g < L * M; g += blockDim.x) {
      const int l = g / M, j = g - l * M;
      const float2* src = in + (long)l * ld;
      float2* dst = out + (long)l * ld;
      const int k = j % Ns;
      float2 v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r)
        if (r < R) v[r] = src[j + r * M];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < 8; ++r)
          if (r < R) {
            float2 w = tw[k * r * tstep];
            if (INV) w.y = -w.y;
            v[r] = cmul(v[r], w);
          }
      }
      gen_butterfly<INV>(R, v);
      const int base = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < 8; ++r)
        if (r < R) dst[base + r * Ns] = v[r];
    }
    __syncthreads();
    float2* t = in;
    in = out;
    out = t;
    Ns *= R;
  }
  return in;
}

// ---- the same line FFT with a compile-time plan (the sides in use: the
// stage radices, spans and strides become constants, so the index arithmetic
// needs no runtime division and each butterfly no radix switch) ----
struct GenPlanC {
  int nst;
  int radix[16];
};

constexpr GenPlanC gen_plan_c(int N) {  // the radix order of gen_plan
  GenPlanC p{0, {}};
  int m = N;
  while (m % 5 == 0) { p.radix[p.nst++] = 5; m /= 5; }
  while (m % 3 == 0) { p.radix[p.nst++] = 3; m /= 3; }
  while (m % 8 == 0) { p.radix[p.nst++] = 8; m /= 8; }
  while (m % 4 == 0) { p.radix[p.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p.radix[p.nst++] = 2; m /= 2; }
  return p;
}

template <int N>
struct GenPlanOf {
  static constexpr GenPlanC P = gen_plan_c(N);
};

template <bool INV, int R>
__device__ __forceinline__ void gen_butterfly_t(float2 (&v)[8]) {
  if constexpr (R == 8)
    dft8<INV>(v);
  else if constexpr (R == 4)
    dft4<INV>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 5)
    dft5<INV>(v[0], v[1], v[2], v[3], v[4]);
  else if constexpr (R == 3)
    dft3<INV>(v[0], v[1], v[2]);
  else
    dft2<INV>(v[0], v[1]);
}

// Per-stage twiddle tables: the stage of span NS and radix R reads
// w^(k r N / (NS R)) for k < NS, 1 <= r < R from st[NS - 1 + (r - 1) NS + k]
// (consecutive k on consecutive threads: distinct banks, where the plain
// table's stride k r N / (NS R) put many k on one bank).  The stage tables
// fill N - 1 entries in all (the spans telescope: sum (NS R - NS) = N - 1).
template <int N, int ST, int NS>
__device__ __forceinline__ void gen_stage_twiddles(float2* st, const float2* __restrict__ gtw) {
  if constexpr (ST < GenPlanOf<N>::P.nst) {
    constexpr int R = GenPlanOf<N>::P.radix[ST];
    constexpr int tstep = N / (NS * R);
    if constexpr (NS > 1)
      for (int i = threadIdx.x; i < NS * (R - 1); i += blockDim.x) {
        const int r = 1 + i / NS, k = i - (r - 1) * NS;
        st[NS - 1 + i] = gtw[k * r * tstep];
      }
    gen_stage_twiddles<N, ST + 1, NS * R>(st, gtw);
  }
}

template <bool INV, int N, int ST, int NS>
__device__ __forceinline__ float2* gen_stages_t(float2* in, float2* out, int L, int ld, const float2* st) {
  if constexpr (ST >= GenPlanOf<N>::P.nst) {
    return in;
  } else {
    constexpr int R = GenPlanOf<N>::P.radix[ST];
    constexpr int M = N / R;
    for (int g = threadIdx.x; g < L * M; g += blockDim.x) {
      const int l = g / M, j = g - l * M;
      const float2* src = in + l * ld;
      float2* dst = out + l * ld;
      const int k = j % NS;
      float2 v[8];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = src[j + r * M];
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = st[NS - 1 + (r - 1) * NS + k];
          if (INV) w.y = -w.y;
          v[r] = cmul(v[r], w);
        }
      }
      gen_butterfly_t<INV, R>(v);
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) dst[base + r * NS] = v[r];
    }
    __syncthreads();
    return gen_stages_t<INV, N, ST + 1, NS * R>(out, in, L, ld, st);
  }
}

// Twiddles into shared memory: the per-stage tables (NT > 0) or the plain
// table w^t, t < N (plan read at run time).
template <int NT>
__device__ __forceinline__ void gen_load_twiddles(float2* tw, int N, const float2* __restrict__ gtw) {
  if constexpr (NT > 0)
    gen_stage_twiddles<NT, 0, 1>(tw, gtw);
  else
    for (int t = threadIdx.x; t < N; t += blockDim.x) tw[t] = gtw[t];
}

// Line FFT with the plan fixed at compile time (NT > 0, tw: the stage tables)
// or read at run time (tw: the plain table).
template <bool INV, int NT>
__device__ __forceinline__ float2* gen_lines(float2* x, float2* y, int L, int ld, const GenPlan& p,
                                             const float2* tw) {
  if constexpr (NT > 0)
    return gen_stages_t<INV, NT, 0, 1>(x, y, L, ld, tw);
  else
    return gen_fft_lines<INV>(x, y, L, ld, p, tw);
}

// ---- rows (c axis) ----
constexpr int GR_LINES = 2;     // lines per CTA
constexpr int GR_THREADS = 256;

struct GenRowsArgs {
  int mode;               // 0 forward (imag * alpha), 1 inverse plain, 2 inverse + HII filter (K radii),
                          // 3 inverse + halo pair filter
  const float2* in;       // modes 0, 2, 3: source box; mode 1: the box (in place)
  float2* out;            // mode 0: destination; mode 1: == in
  const float* alpha;     // mode 0 (may be null)
  Batch bt;               // mode 2
  HfBatch hb;             // mode 3
};

template <int NT>
__global__ void __launch_bounds__(GR_THREADS) k_gen_rows(GenRowsArgs ga, GenPlan p, const float2* __restrict__ gtw) {
  extern __shared__ float2 gsm[];
  const int N = NT > 0 ? NT : p.N;
  float2* tw = gsm;                       // N
  float2* zs = gsm + N;                   // GR_LINES x N: spectrum rows (filter modes)
  float2* b0 = zs + GR_LINES * N;         // GR_LINES x N
  float2* b1 = b0 + GR_LINES * N;         // GR_LINES x N
  gen_load_twiddles<NT>(tw, N, gtw);
  const long row0 = (long)blockIdx.x * GR_LINES;
  const long nrows = (long)N * N;
  const int L = (int)(row0 + GR_LINES <= nrows ? GR_LINES : nrows - row0);
  const float alpha = (ga.mode == 0 && ga.alpha) ? fabsf(*ga.alpha) : 1.0f;
  // load
  for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
    const int l = t / N, c = t - l * N;
    float2 v = ga.in[(row0 + l) * N + c];
    if (ga.mode == 0) v.y *= alpha;
    (ga.mode >= 2 ? zs : b0)[l * N + c] = v;
  }
  __syncthreads();
  if (ga.mode <= 1) {
    float2* r = ga.mode == 0 ? gen_lines<false, NT>(b0, b1, L, N, p, tw) : gen_lines<true, NT>(b0, b1, L, N, p, tw);
    for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
      const int l = t / N, c = t - l * N;
      ga.out[(row0 + l) * N + c] = r[l * N + c];
    }
    return;
  }
  const int K = ga.mode == 2 ? ga.bt.K : ga.hb.K;
  for (int k = 0; k < K; ++k) {
    for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
      const int l = t / N, c = t - l * N;
      const long row = row0 + l;
      const int a = (int)(row / N), b = (int)(row % N);
      const int ka = kfreq(a, N), kb = kfreq(b, N), kc = kfreq(c, N);
      const float kmag = sqrtf((float)(ka * ka + kb * kb + kc * kc));
      const float2 z = zs[l * N + c];
      if (ga.mode == 2) {
        const float w = w_tophat(ga.bt.r[k].dkR * kmag);
        b0[l * N + c] = filter_mul(z, w);
      } else {
        const HfPair& pr = ga.hb.p[k];
        const float wa = ga.hb.scale * w_tophat(pr.dkRa * kmag);
        const float wb = pr.bits_b ? ga.hb.scale * w_tophat(pr.dkRb * kmag) : 0.0f;
        b0[l * N + c] = make_float2(z.x * wa - z.y * wb, z.x * wb + z.y * wa);
      }
    }
    __syncthreads();
    float2* r = gen_lines<true, NT>(b0, b1, L, N, p, tw);
    float2* dst = ga.mode == 2 ? ga.bt.r[k].work : ga.hb.p[k].work;
    for (int t = threadIdx.x; t < L * N; t += blockDim.x) {
      const int l = t / N, c = t - l * N;
      dst[(row0 + l) * N + c] = r[l * N + c];
    }
    __syncthreads();
  }
}

// ---- columns (b or a axis) ----
constexpr int GC_THREADS = 256;

struct GenColsArgs {
  int axis;                 // 1 = b, 0 = a
  int inverse;
  int epi;                  // 0 none (store back), 1 HII centre test + first hit, 2 halo thresholds
  float2* box0;             // single box, or null: the batch's boxes
  Batch bt;                 // epi 0 (box0 null) and epi 1
  HfBatch hb;               // epi 2
  uint8_t* rc;              // epi 1
  const float* alpha;       // epi 1
};

__host__ __device__ __forceinline__ int gen_cw(int N) { return (N <= 600 && N % 16 == 0) ? 16 : 8; }

// Lines in shared memory have a stride ld = 2 (mod 16) float2: the
// transposing load and store (consecutive threads on CW consecutive columns of
// a few rows) then meet distinct banks.
__host__ __device__ __forceinline__ int gen_ld(int N) { return N + ((18 - N % 16) % 16); }

template <int NT, int TH>
__global__ void __launch_bounds__(TH) k_gen_cols(GenColsArgs ga, GenPlan p, const float2* __restrict__ gtw) {
  extern __shared__ float2 gsm[];
  const int N = NT > 0 ? NT : p.N;
  const int CW = gen_cw(N);
  const int ld = gen_ld(N);
  float2* tw = gsm;
  float2* b0 = gsm + N;            // CW lines of N, stride ld
  float2* b1 = b0 + CW * ld;
  uint8_t* hit = reinterpret_cast<uint8_t*>(b1 + CW * ld);  // CW x N (epi 1)
  gen_load_twiddles<NT>(tw, N, gtw);
  const int nblk = N / CW;
  const int outer = blockIdx.x / nblk;
  const int c0 = (blockIdx.x % nblk) * CW;
  const long stride = ga.axis == 1 ? (long)N : (long)N * N;
  const long base = (ga.axis == 1 ? (long)outer * N * N : (long)outer * N) + c0;
  const int nbox = ga.epi == 2 ? ga.hb.K : (ga.box0 ? 1 : ga.bt.K);
  if (ga.epi == 1)
    for (int t = threadIdx.x; t < CW * N; t += blockDim.x) hit[t] = RC_NONE;
  float alpha = 1.0f;
  if (ga.epi == 1) alpha = *ga.alpha;
  for (int k = 0; k < nbox; ++k) {
    float2* box = ga.epi == 2 ? ga.hb.p[k].work : (ga.box0 ? ga.box0 : ga.bt.r[k].work);
    __syncthreads();  // previous use of b0/b1 (and the twiddles on k = 0)
    for (int t = threadIdx.x; t < CW * N; t += blockDim.x) {
      const int row = t / CW, col = t - row * CW;
      b0[col * ld + row] = box[base + (long)row * stride + col];
    }
    __syncthreads();
    float2* r = ga.inverse ? gen_lines<true, NT>(b0, b1, CW, ld, p, tw) : gen_lines<false, NT>(b0, b1, CW, ld, p, tw);
    if (ga.epi == 0) {
      for (int t = threadIdx.x; t < CW * N; t += blockDim.x) {
        const int row = t / CW, col = t - row * CW;
        box[base + (long)row * stride + col] = r[col * ld + row];
      }
    } else if (ga.epi == 1) {
      const int ridx = ga.bt.r[k].ridx;
      for (int t = threadIdx.x; t < CW * N; t += blockDim.x) {
        const int row = t / CW, col = t - row * CW;
        if (is_centre(r[col * ld + row], alpha, ga.bt.zmul) && ridx < hit[t]) hit[t] = (uint8_t)ridx;
      }
    } else {
      // a-axis rows a: the CW cells (a, outer = b, c0 .. c0 + CW - 1) are one
      // aligned byte (CW = 8) or half-word (CW = 16) of each bit set
      const HfPair& pr = ga.hb.p[k];
      for (int row = threadIdx.x; row < N; row += blockDim.x) {
        uint32_t ma = 0, mb = 0;
        for (int col = 0; col < CW; ++col) {
          const float2 v = r[col * ld + row];
          ma |= (v.x > pr.thr_a ? 1u : 0u) << col;
          mb |= (v.y > pr.thr_b ? 1u : 0u) << col;
        }
        const long t = base + (long)row * stride;  // first cell of the run
        if (CW == 16) {
          reinterpret_cast<uint16_t*>(pr.bits_a)[t >> 4] = (uint16_t)ma;
          if (pr.bits_b) reinterpret_cast<uint16_t*>(pr.bits_b)[t >> 4] = (uint16_t)mb;
        } else {
          reinterpret_cast<uint8_t*>(pr.bits_a)[t >> 3] = (uint8_t)ma;
          if (pr.bits_b) reinterpret_cast<uint8_t*>(pr.bits_b)[t >> 3] = (uint8_t)mb;
        }
      }
    }
  }
  if (ga.epi == 1) {
    __syncthreads();
    for (int t = threadIdx.x; t < CW * N; t += blockDim.x) {
      const int row = t / CW, col = t - row * CW;
      const uint8_t h = hit[t];
      if (h != RC_NONE) {
        const long idx = base + (long)row * stride + col;
        if (h < ga.rc[idx]) ga.rc[idx] = h;
      }
    }
  }
}

// ---- host side ----
bool gen_supported(int N) {
  if (N < 24 || N > 1280 || N % 8) return false;  // 1280: the column tile's shared memory
  int m = N;
  for (int f : {2, 3, 5})
    while (m % f == 0) m /= f;
  return m == 1;
}

GenPlan gen_plan(int N) {
  GenPlan p;
  p.N = N;
  p.nst = 0;
  int m = N;
  while (m % 5 == 0) { p.radix[p.nst++] = 5; m /= 5; }
  while (m % 3 == 0) { p.radix[p.nst++] = 3; m /= 3; }
  while (m % 8 == 0) { p.radix[p.nst++] = 8; m /= 8; }
  while (m % 4 == 0) { p.radix[p.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p.radix[p.nst++] = 2; m /= 2; }
  return p;
}

static size_t rows_smem(int N) { return (size_t)(N + 3 * GR_LINES * N) * sizeof(float2); }
static size_t cols_smem(int N) {
  return (size_t)(N + 2 * gen_cw(N) * gen_ld(N)) * sizeof(float2) + (size_t)gen_cw(N) * N;
}

// Sides with a compile-time plan: the reference's defaults (600, 1200) and the
// sides of the reference fixtures that exercise this code (40, 120); others
// run the same kernels with the plan read at run time.  The large sides get
// 512-thread column CTAs.
#define SF21_GEN_SIDES(X) X(40, 256) X(120, 256) X(600, 512) X(1200, 512)

template <int NT, int TH>
static cudaError_t setup_t(int N) {
  cudaError_t e = cudaFuncSetAttribute(k_gen_rows<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem(N));
  if (e) return e;
  return cudaFuncSetAttribute(k_gen_cols<NT, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cols_smem(N));
}

cudaError_t gen_setup(int N) {
  switch (N) {
#define SF21_GEN_CASE(n, th) \
  case n:                    \
    return setup_t<n, th>(N);
    SF21_GEN_SIDES(SF21_GEN_CASE)
#undef SF21_GEN_CASE
    default:
      return setup_t<0, GC_THREADS>(N);
  }
}

template <int NT>
static cudaError_t rows_t(const GenRowsArgs& ga, const GenPlan& p, const float2* tw, cudaStream_t st) {
  const long nrows = (long)p.N * p.N;
  k_gen_rows<NT><<<(unsigned)((nrows + GR_LINES - 1) / GR_LINES), GR_THREADS, rows_smem(p.N), st>>>(ga, p, tw);
  return cudaGetLastError();
}

static cudaError_t rows(const GenRowsArgs& ga, const GenPlan& p, const float2* tw, cudaStream_t st) {
  switch (p.N) {
#define SF21_GEN_CASE(n, th) \
  case n:                    \
    return rows_t<n>(ga, p, tw, st);
    SF21_GEN_SIDES(SF21_GEN_CASE)
#undef SF21_GEN_CASE
    default:
      return rows_t<0>(ga, p, tw, st);
  }
}

template <int NT, int TH>
static cudaError_t cols_t(const GenColsArgs& ga, const GenPlan& p, const float2* tw, cudaStream_t st) {
  const int N = p.N;
  k_gen_cols<NT, TH><<<(unsigned)((long)N * (N / gen_cw(N))), TH, cols_smem(N), st>>>(ga, p, tw);
  return cudaGetLastError();
}

static cudaError_t cols(const GenColsArgs& ga, const GenPlan& p, const float2* tw, cudaStream_t st) {
  switch (p.N) {
#define SF21_GEN_CASE(n, th) \
  case n:                    \
    return cols_t<n, th>(ga, p, tw, st);
    SF21_GEN_SIDES(SF21_GEN_CASE)
#undef SF21_GEN_CASE
    default:
      return cols_t<0, GC_THREADS>(ga, p, tw, st);
  }
}

cudaError_t launch_gen_fwd_rows(const GenPlan& p, const float2* in, float2* out, const float* alpha, const float2* tw,
                                cudaStream_t st) {
  GenRowsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.mode = 0;
  ga.in = in;
  ga.out = out;
  ga.alpha = alpha;
  return rows(ga, p, tw, st);
}

cudaError_t launch_gen_inv_rows_plain(const GenPlan& p, float2* box, const float2* tw, cudaStream_t st) {
  GenRowsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.mode = 1;
  ga.in = box;
  ga.out = box;
  return rows(ga, p, tw, st);
}

cudaError_t launch_gen_inv_rows_filter(const GenPlan& p, const float2* spec, const Batch& bt, const float2* tw,
                                       cudaStream_t st) {
  GenRowsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.mode = 2;
  ga.in = spec;
  ga.bt = bt;
  return rows(ga, p, tw, st);
}

cudaError_t launch_gen_hf_rows_filter(const GenPlan& p, const float2* spec, const HfBatch& hb, const float2* tw,
                                      cudaStream_t st) {
  GenRowsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.mode = 3;
  ga.in = spec;
  ga.hb = hb;
  return rows(ga, p, tw, st);
}

cudaError_t launch_gen_cols(const GenPlan& p, float2* box, const Batch& bt, int axis, bool inverse, const float2* tw,
                            cudaStream_t st) {
  GenColsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.axis = axis;
  ga.inverse = inverse;
  ga.epi = 0;
  ga.box0 = box;
  ga.bt = bt;
  return cols(ga, p, tw, st);
}

cudaError_t launch_gen_cols_a_test(const GenPlan& p, const Batch& bt, uint8_t* rc, const float* alpha,
                                   const float2* tw, cudaStream_t st) {
  GenColsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.axis = 0;
  ga.inverse = 1;
  ga.epi = 1;
  ga.bt = bt;
  ga.rc = rc;
  ga.alpha = alpha;
  return cols(ga, p, tw, st);
}

cudaError_t launch_gen_hf_cols(const GenPlan& p, const HfBatch& hb, int axis, bool thresholds, const float2* tw,
                               cudaStream_t st) {
  GenColsArgs ga;
  memset(&ga, 0, sizeof ga);
  ga.axis = axis;
  ga.inverse = 1;
  ga.epi = thresholds ? 2 : 0;
  ga.hb = hb;
  // the plain pass walks the pair boxes as a Batch
  ga.bt.K = hb.K;
  for (int k = 0; k < hb.K; ++k) ga.bt.r[k].work = hb.p[k].work;
  return cols(ga, p, tw, st);
}

}  // namespace sf21
