// Column-block-major layout of the work boxes (kernels_cb.cu, kernels_hf.cu):
//     index(a, b, c) = ((c / CW) N + a) N + b) CW + c mod CW,
// one slab of N^2 x CW values per column block, and the CTA shapes of the
// passes over it.
#pragma once
#include "fft_line.cuh"

namespace sf21 {

template <int N>
struct CbGeom {
  static constexpr int CW = (N <= 512) ? 16 : 8;  // columns per block (CW * 8 bytes per run)
  static constexpr int NBLK = N / CW;
  static constexpr int RT = N / 8;                // threads per row (c-axis pass)
  static constexpr int ROWS = (256 / RT) > 0 ? (256 / RT) : 1;
  static constexpr int RTHREADS = RT * ROWS;
};

template <int N>
__device__ __forceinline__ long cb_index(int a, int b, int c) {
  using G = CbGeom<N>;
  return (((long)(c / G::CW) * N + a) * N + b) * G::CW + (c % G::CW);
}

// b- and a-axis passes: one CTA per tile of a whole column block.
// With 16 columns a warp covers 16 lines x 2 threads, whose shared-memory
// exchanges of the line FFT are free of bank conflicts.  (Half blocks of 8
// columns, two CTAs per SM, measured slower even with a conflict-free
// exchange padding.)
template <int N>
struct KGeom {
  static constexpr int KW = CbGeom<N>::CW;  // columns per CTA
  static constexpr int THREADS = KW * (N / 8);
  static constexpr int LS = LineGeom<N>::LS;  // float2 per exchange line
  static constexpr size_t SMEM = (size_t)(N + 2 * KW * LS) * sizeof(float2);  // two lines each
  static constexpr int PER_SM = THREADS <= 512 ? 2 : 1;
};

}  // namespace sf21
