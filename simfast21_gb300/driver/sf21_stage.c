/*
 * Host side of the HII stage for the sf21_hii driver (see sf21_stage.h).
 */
#define _POSIX_C_SOURCE 200809L
#include "sf21_stage.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const double kPI = 3.1415926535897932385E0; /* Input_variables.h:10 */

int sf21_read_params(const char *basedir, sf21_stage_params *p) {
  char fname[1024], line[256], first[100], third[100];
  memset(p, 0, sizeof(*p));
  snprintf(fname, sizeof fname, "%s/simfast21.ini", basedir);
  FILE *f = fopen(fname, "r");
  if (!f) return 1;
  double sim_length = 0, rmax_mpc = 0;
  while (fgets(line, sizeof line, f) != NULL) {
    if (line[0] == '#' || line[0] == '\n') continue;
    char *eq = strchr(line, '=');
    if (!eq) { fclose(f); return 2; }            /* "Wrong format!" (:40) */
    *eq = ' ';
    if (sscanf(line, "%99s %99s", first, third) != 2) { fclose(f); return 2; }  /* (:42-43) */
    if (!strcmp(first, "nthreads")) p->nthreads = atoi(third);
    else if (!strcmp(first, "dz")) p->dz = atof(third);
    else if (!strcmp(first, "zmax")) p->zmax = atof(third);
    else if (!strcmp(first, "zmin")) p->zmin = atof(third);
    else if (!strcmp(first, "sim_length")) sim_length = atof(third);
    else if (!strcmp(first, "N_halo")) p->N_halo = atoi(third);
    else if (!strcmp(first, "N_smoothed")) p->N_smooth = atoi(third);
    else if (!strcmp(first, "hubble")) p->hubble = atof(third);
    else if (!strcmp(first, "fesc")) p->fesc = atof(third);
    else if (!strcmp(first, "Ion_cutoff")) p->xHlim = atof(third);
    else if (!strcmp(first, "bubble_Rmax")) rmax_mpc = atof(third);
    else if (!strcmp(first, "bubble_Nbins")) p->bubble_Nbins = atoi(third);
    else if (!strcmp(first, "use_SFR")) {
      if (!strcmp(third, "T")) p->use_SFR = 1;
      if (!strcmp(third, "F")) p->use_SFR = 0;
    } else if (!strcmp(first, "hii_param_sets")) {
      snprintf(p->param_sets_file, sizeof p->param_sets_file, "%s", third);
    }
  }
  fclose(f);
  /* Input_variables.c:121-133 */
  p->L = sim_length * p->hubble;
  p->bubble_Rmax = rmax_mpc * p->hubble;
  if (p->bubble_Rmax > p->L / 2.) p->bubble_Rmax = p->L / 2.;
  p->zmin = p->zmax - p->dz * (double)ceil((p->zmax - p->zmin) / p->dz);
  (void)kPI;
  return 0;
}

int sf21_read_box(const char *path, float *buf, long n) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  size_t got = fread(buf, sizeof(float), (size_t)n, f);
  fclose(f);
  return got == (size_t)n ? 0 : 2;
}

int sf21_write_box(const char *path, const float *buf, long n) {
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  size_t put = fwrite(buf, sizeof(float), (size_t)n, f);
  fclose(f);
  return put == (size_t)n ? 0 : 2;
}

/* Rion(M, z), user_functions.c:40-47 */
static double rion_of(float m, double z) {
  const double c1 = 1.575e39, c2 = 9.367608e+07, c3 = 0.44, c4 = 2.27044695e+00;
  double t1 = c1 * m * pow((1.0 + z), c4);
  double t2 = pow((m / c2), c3);
  double t3 = exp(-pow((c2 / m), 3.0));
  return t1 * t2 * t3 / 1.e+45;
}

static long wrap(long x, long n) {
  x = x % n;
  if (x < 0) x += n;
  return x;
}

/* cloud-in-cell of one value, the reference's corner order (auxiliary.c:761-808) */
static void cic(float x1, float y1, float z1, float v, float *map, long N) {
  long x = (long)x1, y = (long)y1, z = (long)z1;
  x1 -= x;
  y1 -= y;
  z1 -= z;
  for (long a = 0; a < 2; a++)
    for (long b = 0; b < 2; b++)
      for (long c = 0; c < 2; c++) {
        x += a; y += b; z += c;
        if (x1 < 0.0) { x = x - 1; x1 = fabsf(x1); }
        if (y1 < 0.0) { y = y - 1; y1 = fabsf(y1); }
        if (z1 < 0.0) { z = z - 1; z1 = fabsf(z1); }
        x = wrap(x, N); y = wrap(y, N); z = wrap(z, N);
        if (a == 1) x1 = 1.0 - x1;
        if (b == 1) y1 = 1.0 - y1;
        if (c == 1) z1 = 1.0 - z1;
        map[x * N * N + y * N + z] += (1.0 - x1) * (1.0 - y1) * (1.0 - z1) * v;
        x -= a; y -= b; z -= c;
        if (a == 1) x1 = 1.0 - x1;
        if (b == 1) y1 = 1.0 - y1;
        if (c == 1) z1 = 1.0 - z1;
      }
}

int sf21_halo_rion_box(const char *path, double z, const sf21_stage_params *p, float *out) {
  typedef struct { float Mass, x, y, z; } halo_t; /* auxiliary.h:13-17 */
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  long nh = 0;
  if (fread(&nh, sizeof(long), 1, f) != 1 || nh < 0) { fclose(f); return 2; }
  halo_t *h = malloc(sizeof(halo_t) * (size_t)(nh ? nh : 1));
  if (!h) { fclose(f); return 3; }
  if (fread(h, sizeof(halo_t), (size_t)nh, f) != (size_t)nh) { free(h); fclose(f); return 2; }
  fclose(f);
  const long Nh = p->N_halo, Ns = p->N_smooth;
  if (Ns > Nh) { free(h); return 4; } /* auxiliary.c:651-654 */
  float *fine = calloc((size_t)(Nh * Nh * Nh), sizeof(float));
  if (!fine) { free(h); return 3; }
  for (long i = 0; i < nh; i++) cic(h[i].x, h[i].y, h[i].z, (float)rion_of(h[i].Mass, z), fine, Nh);
  free(h);
  long sm = (long)roundf((1.0 * Nh) / Ns);
  if (Ns * sm > Nh) sm = sm - 1;
  const double sm3 = 1.0 * sm * sm * sm;
  for (long i = 0; i < Ns; i++)
    for (long j = 0; j < Ns; j++)
      for (long q = 0; q < Ns; q++) {
        double av = 0.0;
        for (long a = 0; a < sm; a++)
          for (long b = 0; b < sm; b++)
            for (long c = 0; c < sm; c++) av += fine[(i * sm + a) * Nh * Nh + (j * sm + b) * Nh + (q * sm + c)];
        out[i * Ns * Ns + j * Ns + q] = (float)(av / sm3);
      }
  free(fine);
  return 0;
}
