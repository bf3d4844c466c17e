/*
 * Single- and double-precision 3D real FFTs behind the FFTW3 API (see
 * fftw3.h): the body in fftw_shim_body.h is compiled once per precision.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY: used to build the reference's own
 * get_HIIbubbles.c (oracle/_ref) and the CPU restatement oracle/hii_oracle.c.
 * It never ships in the GPU product library.
 *
 * Algorithm (the published mixed-radix Stockham autosort DFT):
 *   for each radix R of n (4,2,3,5, then any odd prime), with Ns = product
 *   of the radices already applied:
 *     v[r] = x[j + r n/R] * w^(r (j mod Ns) n/(Ns R)),  r = 0..R-1
 *     V = DFT_R(v)
 *     y[(j/Ns) Ns R + (j mod Ns) + r Ns] = V[r]
 * Arithmetic is in the API's precision (float for fftwf_, double for
 * fftw_), twiddles are computed in double and rounded once.
 * r2c/c2r along the last axis use the half-length complex packing
 * (x[2m] + i x[2m+1]) for even n2.  The other axes are complex transforms
 * over gathered column blocks.  OpenMP threads split the independent lines
 * (the reference's FFTW is OpenMP-threaded as well, makefile:8,14).
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fftw3.h"

#define SHIM_PI 3.14159265358979323846

#define COLBLK 16

static int g_nthreads = 1; /* shared by both precisions, as FFTW's threads */

#define SHIM_CAT2(a, b) a##b
#define SHIM_CAT(a, b) SHIM_CAT2(a, b)
#define S(x) SHIM_CAT(x, SHIM_SUF)
#define API(x) SHIM_CAT(SHIM_PFX, x)

/* single precision: fftwf_* */
#define SREAL float
#define SCPX cpx_sf
#define SPLAN sf21_shim_plan_s
#define SPLAN_T fftwf_plan
#define SCOMPLEX_T fftwf_complex
#define SHIM_SUF _sf
#define SHIM_PFX fftwf_
#include "fftw_shim_body.h"
#undef SREAL
#undef SCPX
#undef SPLAN
#undef SPLAN_T
#undef SCOMPLEX_T
#undef SHIM_SUF
#undef SHIM_PFX

/* double precision: fftw_* (the reference's t21.c, :104-111) */
#define SREAL double
#define SCPX cpx_sd
#define SPLAN sf21_shim_plan_d
#define SPLAN_T fftw_plan
#define SCOMPLEX_T fftw_complex
#define SHIM_SUF _sd
#define SHIM_PFX fftw_
#include "fftw_shim_body.h"
