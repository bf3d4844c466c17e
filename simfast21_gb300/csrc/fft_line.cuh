// Batched 1D complex FFT of a power-of-two length N (16 <= N <= 1024) held
// by N/8 threads of a CTA, 8 elements per thread.
//
// Stockham autosort with radix-8 stages and one radix-2 or radix-4 tail:
//   stage with Ns = product of earlier radices:
//     v[r] = x[j + r N/R] * w^((j mod Ns) r N/(Ns R)),   V = DFT_R(v),
//     x'[(j/Ns) Ns R + (j mod Ns) + r Ns] = V[r]
// The first stage takes its inputs from registers and the last stage leaves
// its outputs in registers, in the same ownership: on entry and on exit
// thread j holds elements j + r N/8 (r = 0..7) of its line, so global loads
// and stores of a line are coalesced across the threads of a warp.  Only the
// exchanges between stages go through shared memory (one float2 per element,
// padded index n + n/16 to keep the strided stage stores at most 2-way
// bank-conflicted).
//
// Twiddles come from a table computed in double on the host and rounded once,
// laid out stage by stage so that the lanes of a warp read consecutive
// entries (no shared-memory bank conflicts): for the radix-8 stage with
// stride Ns the entry (r - 1) Ns + (j mod Ns) holds w^((j mod Ns) r N/(8 Ns)),
// for the radix-4 tail (r - 1) N/4 + j4 holds w^(j4 r), for the radix-2 tail
// j2 holds w^j2, with w = exp(-2 pi i / N) (twiddle_layout() below gives the
// offsets); the inverse transform uses the conjugates.  Transforms are
// unnormalised (forward sign -1, inverse +1), the FFTW convention the
// reference relies on (get_HIIbubbles.c:110-183).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace sf21 {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

__device__ __forceinline__ int padx(int n) { return n + (n >> 4); }

template <int N>
struct LineGeom {
  static constexpr int LOG = ilog2c(N);
  static constexpr int T = N / 8;                    // threads per line
  static constexpr int LS = N + N / 16 + 1;          // float2 per line (odd)
  static_assert((N & (N - 1)) == 0 && N >= 16 && N <= 1024, "N must be a power of two in [16, 1024]");
};

// CTA shapes of the line passes: contiguous-axis rows (T threads per row,
// ROWS rows per CTA) and strided-axis tiles (N rows x CW contiguous columns).
template <int N>
struct RowGeom {
  static constexpr int T = N / 8;
  static constexpr int ROWS = (256 / T) > 0 ? (256 / T) : 1;  // rows per CTA
  static constexpr int THREADS = T * ROWS;
};

template <int N>
struct ColGeom {
  static constexpr int CW = (N <= 512) ? 16 : 8;  // columns (contiguous c) per tile
  static constexpr int THREADS = CW * (N / 8);
};

template <int N>
__device__ __forceinline__ void load_twiddles(float2* stw, const float2* __restrict__ gtw) {
  for (int t = threadIdx.x; t < N; t += blockDim.x) stw[t] = gtw[t];
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// Every product that feeds an addition in the line transforms is written as
// an explicit fused multiply-add (the other product rounded on its own):
// left to the compiler, the contraction may differ between two kernels that
// inline the same transform, and their outputs would then differ in the last
// bit.  Written out, every kernel built on these transforms gets the same bits.
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -__fmul_rn(a.y, b.y)), fmaf(a.x, b.y, __fmul_rn(a.y, b.x)));
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  float2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  float2 t2 = cadd(a1, a3), t3 = mul_mi<INV>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2 (&v)[8]) {
  const float h = 0.70710678118654752440f;
  // DIT: E = DFT4(v0,v2,v4,v6), O = DFT4(v1,v3,v5,v7)
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  // twiddles w8^k, w8 = exp(-/+ i pi/4): w8 o = h s with s a sum of the
  // parts of o, applied as e + h s and e - h s (explicit fused multiply-adds)
  float2 s1, s3, w2o;
  if (!INV) {
    s1 = make_float2(o1.x + o1.y, o1.y - o1.x);
    w2o = make_float2(o2.y, -o2.x);
    s3 = make_float2(o3.y - o3.x, -(o3.x + o3.y));
  } else {
    s1 = make_float2(o1.x - o1.y, o1.x + o1.y);
    w2o = make_float2(-o2.y, o2.x);
    s3 = make_float2(-(o3.x + o3.y), o3.x - o3.y);
  }
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = make_float2(fmaf(h, s1.x, e1.x), fmaf(h, s1.y, e1.y));
  v[5] = make_float2(fmaf(-h, s1.x, e1.x), fmaf(-h, s1.y, e1.y));
  v[2] = cadd(e2, w2o);
  v[6] = csub(e2, w2o);
  v[3] = make_float2(fmaf(h, s3.x, e3.x), fmaf(h, s3.y, e3.y));
  v[7] = make_float2(fmaf(-h, s3.x, e3.x), fmaf(-h, s3.y, e3.y));
}

// Offset of the twiddles of radix-8 stage st (st >= 1) in the table.
__host__ __device__ constexpr int tw_stage_off(int st) {
  int off = 0, ns = 8;
  for (int s = 1; s < st; ++s) {
    off += 7 * ns;
    ns *= 8;
  }
  return off;
}
// Offset of the tail twiddles (after the Q radix-8 stages).
__host__ __device__ constexpr int tw_tail_off(int N) { return tw_stage_off(ilog2c(N) / 3); }

template <bool INV>
__device__ __forceinline__ float2 twid(const float2* tw, int t) {
  float2 w = tw[t];
  if (INV) w.y = -w.y;
  return w;
}

// One line: s = this line's shared-memory slice (LineGeom<N>::LS float2),
// tw = shared or global twiddle table of N entries, j = thread index in line.
// All threads of the CTA must call it together (it synchronises the CTA).
template <int N, bool INV>
__device__ __forceinline__ void fft_line(float2 (&v)[8], float2* s, const float2* tw, int j) {
  constexpr int LOG = LineGeom<N>::LOG;
  constexpr int Q = LOG / 3;
  constexpr int RB = LOG % 3;
  constexpr int N8 = N / 8;
  int Ns = 1;
#pragma unroll
  for (int st = 0; st < Q; ++st) {
    if (st > 0) {
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = s[padx(j + r * N8)];
      const int jm = j & (Ns - 1);
      const float2* tws = tw + tw_stage_off(st);
#pragma unroll
      for (int r = 1; r < 8; ++r) v[r] = cmul(v[r], twid<INV>(tws, (r - 1) * Ns + jm));
    }
    dft8<INV>(v);
    const bool keep = (st == Q - 1) && (RB == 0);
    if (!keep) {
      __syncthreads();
      const int base = (j / Ns) * Ns * 8 + (j & (Ns - 1));
#pragma unroll
      for (int r = 0; r < 8; ++r) s[padx(base + r * Ns)] = v[r];
      __syncthreads();
    }
    Ns *= 8;
  }
  if (RB == 1) {
    // radix-2 tail, Ns = N/2: butterflies j2 = j + m N/8, m = 0..3
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int j2 = j + m * N8;
      float2 a = s[padx(j2)];
      float2 b = cmul(s[padx(j2 + N / 2)], twid<INV>(tw + tw_tail_off(N), j2));
      v[m] = cadd(a, b);
      v[m + 4] = csub(a, b);
    }
  } else if (RB == 2) {
    // radix-4 tail, Ns = N/4: butterflies j4 in {j, j + N/8}
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j4 = j + h * N8;
      const float2* twt = tw + tw_tail_off(N);
      float2 a0 = s[padx(j4)];
      float2 a1 = cmul(s[padx(j4 + N / 4)], twid<INV>(twt, j4));
      float2 a2 = cmul(s[padx(j4 + N / 2)], twid<INV>(twt, N / 4 + j4));
      float2 a3 = cmul(s[padx(j4 + 3 * N / 4)], twid<INV>(twt, N / 2 + j4));
      dft4<INV>(a0, a1, a2, a3);
      // outputs j4 + r N/4 -> register j + (2r + h) N/8
      v[0 + h] = a0;
      v[2 + h] = a1;
      v[4 + h] = a2;
      v[6 + h] = a3;
    }
  }
}

// The same with two exchange buffers used in turn (s0, s1: LineGeom<N>::LS
// float2 each): one barrier per exchange instead of two.  A buffer is written
// only after the barrier that follows the last read of it, so when the
// number of exchanges per call is even (N = 128, 256, 512) consecutive calls
// need no barrier between them; for an odd count (FftPP<N>::CALL_SYNC) the
// caller keeps a __syncthreads() before each call.
template <int N>
struct FftPP {
  static constexpr int LOG = LineGeom<N>::LOG;
  static constexpr int Q = LOG / 3;
  static constexpr int RB = LOG % 3;
  static constexpr int EXCH = (RB == 0) ? Q - 1 : Q;  // shared-memory exchanges per call
  static constexpr bool CALL_SYNC = (EXCH % 2) != 0;
};

// Padded exchange indices as one per-thread base plus compile-time offsets
// (identical to padx() of the full index, checked over every N, j and r):
//   padx(j + r N/8)       = padx(j) + r (N/8 + N/128)          (N/8 % 16 == 0)
//   padx(8 j + r)         = 8 j + (j >> 1) + r                  (Ns = 1)
//   padx(b8 + 8 r)        = (j/8) 68 + (j & 7) + 8 r + (r >> 1) (Ns = 8)
//   padx(bNs + r Ns)      = padx(bNs) + r (Ns + Ns/16)          (Ns % 16 == 0)
// with bNs = (j/Ns) 8 Ns + j mod Ns, the store base of the exchange.
template <int N>
__device__ __forceinline__ int pp_load_index(int j, int r) {
  constexpr int N8 = N / 8;
  if constexpr (N8 % 16 == 0) return padx(j) + r * (N8 + N8 / 16);
  else return padx(j + r * N8);
}
template <int Ns>
__device__ __forceinline__ int pp_store_index(int j, int r) {
  if constexpr (Ns == 1) return 8 * j + (j >> 1) + r;
  else if constexpr (Ns == 8) return (j >> 3) * 68 + (j & 7) + 8 * r + (r >> 1);
  else if constexpr (Ns % 16 == 0) return padx((j / Ns) * Ns * 8 + (j & (Ns - 1))) + r * (Ns + Ns / 16);
  else return padx((j / Ns) * Ns * 8 + (j & (Ns - 1)) + r * Ns);
}

template <int N, bool INV>
__device__ __forceinline__ void fft_line_pp(float2 (&v)[8], float2* s0, float2* s1, const float2* tw, int j) {
  constexpr int Q = FftPP<N>::Q;
  constexpr int RB = FftPP<N>::RB;
  constexpr int N8 = N / 8;
  int Ns = 1;
  float2* cur = s0;  // buffer written by the next exchange
#pragma unroll
  for (int st = 0; st < Q; ++st) {
    if (st > 0) {
      float2* prev = (st & 1) ? s0 : s1;  // written by the previous exchange
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = prev[pp_load_index<N>(j, r)];
      const int jm = j & (Ns - 1);
      const float2* tws = tw + tw_stage_off(st);
#pragma unroll
      for (int r = 1; r < 8; ++r) v[r] = cmul(v[r], twid<INV>(tws, (r - 1) * Ns + jm));
    }
    dft8<INV>(v);
    const bool keep = (st == Q - 1) && (RB == 0);
    if (!keep) {
      cur = (st & 1) ? s1 : s0;
      if (st == 0) {
#pragma unroll
        for (int r = 0; r < 8; ++r) cur[pp_store_index<1>(j, r)] = v[r];
      } else if (st == 1) {
#pragma unroll
        for (int r = 0; r < 8; ++r) cur[pp_store_index<8>(j, r)] = v[r];
      } else {
#pragma unroll
        for (int r = 0; r < 8; ++r) cur[pp_store_index<64>(j, r)] = v[r];
      }
      __syncthreads();
    }
    Ns *= 8;
  }
  const float2* s = cur;
  if (RB == 1) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int j2 = j + m * N8;
      float2 a = s[padx(j2)];
      float2 b = cmul(s[padx(j2 + N / 2)], twid<INV>(tw + tw_tail_off(N), j2));
      v[m] = cadd(a, b);
      v[m + 4] = csub(a, b);
    }
  } else if (RB == 2) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j4 = j + h * N8;
      const float2* twt = tw + tw_tail_off(N);
      float2 a0 = s[padx(j4)];
      float2 a1 = cmul(s[padx(j4 + N / 4)], twid<INV>(twt, j4));
      float2 a2 = cmul(s[padx(j4 + N / 2)], twid<INV>(twt, N / 4 + j4));
      float2 a3 = cmul(s[padx(j4 + 3 * N / 4)], twid<INV>(twt, N / 2 + j4));
      dft4<INV>(a0, a1, a2, a3);
      v[0 + h] = a0;
      v[2 + h] = a1;
      v[4 + h] = a2;
      v[6 + h] = a3;
    }
  }
}

// Host: the twiddle table of an N-point line in the layout above (N entries,
// the unused tail is zero).  out[t] = (cos, sin) of the angle, in double.
inline void twiddle_layout(int N, double* re, double* im) {
  const double two_pi = 6.283185307179586476925286766559;
  for (int t = 0; t < N; ++t) re[t] = im[t] = 0.0;
  const int LOG = ilog2c(N), Q = LOG / 3, RB = LOG % 3;
  int Ns = 8;
  for (int st = 1; st < Q; ++st) {
    const int off = tw_stage_off(st);
    for (int r = 1; r < 8; ++r)
      for (int jm = 0; jm < Ns; ++jm) {
        const long e = (long)jm * r * (N / (8 * Ns));
        re[off + (r - 1) * Ns + jm] = cos(-two_pi * (double)e / N);
        im[off + (r - 1) * Ns + jm] = sin(-two_pi * (double)e / N);
      }
    Ns *= 8;
  }
  const int off = tw_tail_off(N);
  if (RB == 2) {
    for (int r = 1; r < 4; ++r)
      for (int j4 = 0; j4 < N / 4; ++j4) {
        re[off + (r - 1) * (N / 4) + j4] = cos(-two_pi * (double)(j4 * r) / N);
        im[off + (r - 1) * (N / 4) + j4] = sin(-two_pi * (double)(j4 * r) / N);
      }
  } else if (RB == 1) {
    for (int j2 = 0; j2 < N / 2; ++j2) {
      re[off + j2] = cos(-two_pi * (double)j2 / N);
      im[off + j2] = sin(-two_pi * (double)j2 / N);
    }
  }
}

}  // namespace sf21
