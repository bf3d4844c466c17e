/*
 * sf21_power3d_f: drop-in for the reference's power-spectrum tool
 * tools/power3d_f.c on one GPU.
 *
 *   sf21_power3d_f Nbytes N1 N2 N3 dl flag input_file [nthreads]
 *
 * Same arguments (nthreads accepted and ignored), same input (raw float or
 * double box, N3 fastest), same text on standard output: the parameter line,
 * the window sum, and one "k P(k)" line per spherical bin.  Only cubic boxes
 * of the library's transform sizes (a power of two from 16 to 1024, or a
 * product of 2, 3 and 5 that 8 divides, from 24 to 1280); anything else exits
 * 1 with a message.  The window is applied on the host
 * in double exactly as the tool does ((float)(value * window),
 * power3d_f.c:134-156) and the sum of its square is taken in the tool's
 * loop order (:121-128); transform and binning run through
 * sf21_hii_power_spectrum.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sf21_hii.h"

static double wind1(long x, long m, int flag) {
  if (flag == 1) return 1 - fabs(x - m / 2.) / m * 2.;
  if (flag == 2) return (1 - ((x - m / 2.) / m * 2.) * ((x - m / 2.) / m * 2.));
  return 1.0;
}

/* the tool's wind(): the product of the three axis factors, left to right */
static double wind3(long i, long j, long p, long m, int flag) {
  if (flag == 0) return 1.0;
  return wind1(i, m, flag) * wind1(j, m, flag) * wind1(p, m, flag);
}

int main(int argc, char **argv) {
  if (argc != 8 && argc != 9) {
    printf("SYNTAX: sf21_power3d_f Nbytes N1 N2 N3 dl flag input_file [nthreads] (output goes to standard output)\n");
    return 1;
  }
  const int bsize = atoi(argv[1]);
  const long N1 = atol(argv[2]), N2 = atol(argv[3]), N3 = atol(argv[4]);
  const double dl = atof(argv[5]);
  const int flag = atoi(argv[6]);
  const char *fname = argv[7];
  const double PI = 3.1415926535897932385E0;
  const double L1 = N1 * dl, L2 = N2 * dl, L3 = N3 * dl;
  double dk = 2.0 * PI / L1;
  if (2.0 * PI / L2 > dk) dk = 2.0 * PI / L2;
  if (2.0 * PI / L3 > dk) dk = 2.0 * PI / L3;
  printf("# Input parameters - Nbytes:%d, N1:%ld,  N2:%ld, N3:%ld, dl:%f, flag:%d, L1:%f, L2:%f, L3:%f, dk:%f, "
         "input file:%s\n", bsize, N1, N2, N3, dl, flag, L1, L2, L3, dk, fname);
  if (N1 != N2 || N2 != N3 || (bsize != 4 && bsize != 8) || !(dl > 0)) {
    printf("sf21_power3d_f: only cubic boxes, Nbytes 4 or 8, dl > 0\n");
    return 1;
  }
  const long N = N1, n3 = N * N * N;
  FILE *fid = fopen(fname, "rb");
  if (!fid) {
    printf("Reading file error...\n");
    return 1;
  }
  void *raw = malloc((size_t)n3 * bsize);
  float *boxw = malloc(sizeof(float) * (size_t)n3);
  if (!raw || !boxw) {
    printf("Mem1 Problem...\n");
    return 1;
  }
  if (fread(raw, bsize, (size_t)n3, fid) != (size_t)n3) {
    printf("Reading file error...\n");
    return 1;
  }
  fclose(fid);
  const long m = N - 1;
  double wsum = 0.;
  for (long i = 0; i < N; i++)
    for (long j = 0; j < N; j++)
      for (long p = 0; p < N; p++) wsum += wind3(i, j, p, m, flag) * wind3(i, j, p, m, flag);
  printf("# Window sum: %E\n", wsum);
  fflush(stdout);
  for (long i = 0; i < N; i++)
    for (long j = 0; j < N; j++)
      for (long p = 0; p < N; p++) {
        const long t = (i * N + j) * N + p;
        const double v = bsize == 4 ? (double)((float *)raw)[t] : ((double *)raw)[t];
        boxw[t] = (float)(v * wind3(i, j, p, m, flag));
      }
  free(raw);

  sf21_hii_set set = {1.0, dl * N / 4.0, 1};
  sf21_hii_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.N = N;
  cfg.N_halo = N;
  cfg.L = dl * N;
  cfg.hubble = 1.0;
  cfg.nsets = 1;
  cfg.sets = &set;
  cfg.kmax = 1;
  cfg.path = 1; /* no radius pipeline is used: skip the tuning */
  sf21_hii_ctx *ctx = NULL;
  if (sf21_hii_create(&cfg, &ctx) != SF21_OK) {
    printf("sf21_power3d_f: %s\n", sf21_hii_last_error(NULL));
    return 1;
  }
  const int cap = (int)(2 * N);
  double *k = malloc(sizeof(double) * cap), *P = malloc(sizeof(double) * cap);
  /* window already applied: flag 0 inside, whose sum of squares is N^3 */
  const int nk = sf21_hii_power_spectrum(ctx, boxw, 0, dl, k, P, cap);
  if (nk < 0) {
    printf("sf21_power3d_f: %s\n", sf21_hii_last_error(ctx));
    return 1;
  }
  printf("# Now calculating power spectum\n");
  printf("# Output: k(units 1/dl)     P(k)(units of input box cell values^2*dl^3)\n");
  const double scale = (double)n3 / wsum;
  for (int b = 0; b < nk; b++) printf("%f   %E\n", b * dk, P[b] * scale);
  sf21_hii_destroy(ctx);
  free(k);
  free(P);
  free(boxw);
  return 0;
}
