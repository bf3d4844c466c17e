/*
 * FFTW3 API subset (single precision, and the double-precision twin used by
 * the reference's t21.c), implemented by fftw_shim.c.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  FFTW3 is not installed in the build
 * container nor on the GPU host, so this header lets the reference's own
 * get_HIIbubbles.c (and the CPU restatement in oracle/hii_oracle.c) compile
 * unchanged.  Only the symbols the HII stage calls are provided:
 *   fftwf_complex, fftwf_plan, fftwf_malloc/free, fftwf_plan_dft_r2c_3d,
 *   fftwf_plan_dft_c2r_3d, fftwf_execute, fftwf_destroy_plan,
 *   fftwf_init_threads, fftwf_plan_with_nthreads, FFTW_MEASURE/ESTIMATE.
 * Call sites mirrored: get_HIIbubbles.c:74-79 (threads), :102-183 (plans),
 * :290-291, :324-325, :372-382, :424-425 (execute).
 *
 * Semantics follow the published FFTW3 interface: row-major n0 x n1 x n2,
 * r2c output n0 x n1 x (n2/2+1), transforms unnormalised, forward sign -1,
 * c2r sign +1; an in-place plan (same array for input and output, as the
 * halo finder's c2r at get_halos.c:143) uses FFTW's padded real layout,
 * rows of 2 (n2/2+1) reals.  FFTW's own version is unpinned (makefile:8-9 links
 * -lfftw3f_omp -lfftw3f with no version), so parity is pinned on the
 * mathematics of the DFT, not on FFTW's rounding.
 */
#ifndef SF21_ORACLE_FFTW3_SHIM_H
#define SF21_ORACLE_FFTW3_SHIM_H

#include <stddef.h>
#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FFTW defines fftwf_complex as the C99 complex type when <complex.h> was
 * included first (get_HIIbubbles.c:19-20 includes it first). */
typedef float _Complex fftwf_complex;

typedef struct sf21_shim_plan_s *fftwf_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)

void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int nthreads);
void fftwf_cleanup_threads(void);
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in,
                                 fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in,
                                 float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);

/* double precision (t21.c:104-111, 222, 243) */
typedef double _Complex fftw_complex;
typedef struct sf21_shim_plan_d *fftw_plan;
void *fftw_malloc(size_t n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
