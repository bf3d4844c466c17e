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
    } else if (!strcmp(first, "omega_matter")) p->omega_m = atof(third);
    else if (!strcmp(first, "omega_baryon")) p->omega_b = atof(third);
    else if (!strcmp(first, "omega_lambda")) p->omega_l = atof(third);
    else if (!strcmp(first, "Vel_comp")) p->vel_comp = atoi(third);
    else if (!strcmp(first, "use_Lya_xrays")) {
      if (!strcmp(third, "T")) p->use_Lya_xrays = 1;
      if (!strcmp(third, "F")) p->use_Lya_xrays = 0;
    } else if (!strcmp(first, "Zminsfr")) p->Zminsfr = atof(third);
    else if (!strcmp(first, "sigma8")) p->sigma8 = atof(third);
    else if (!strcmp(first, "spectral_index")) p->n_index = atof(third);
    else if (!strcmp(first, "critical_overdensity")) p->delta_c = atof(third);
    else if (!strcmp(first, "STa")) p->STa = atof(third);
    else if (!strcmp(first, "STb")) p->STb = atof(third);
    else if (!strcmp(first, "STc")) p->STc = atof(third);
    else if (!strcmp(first, "Use_subgrid")) p->use_sgrid = !strcmp(third, "T");
    else if (!strcmp(first, "halo_Mmin")) p->halo_Mmin = atof(third);
    else if (!strcmp(first, "halo_dlm")) p->halo_dlm = atof(third);
  }
  fclose(f);
  /* Input_variables.c:121-133 */
  p->L = sim_length * p->hubble;
  p->bubble_Rmax = rmax_mpc * p->hubble;
  if (p->bubble_Rmax > p->L / 2.) p->bubble_Rmax = p->L / 2.;
  p->zmin = p->zmax - p->dz * (double)ceil((p->zmax - p->zmin) / p->dz);
  p->Zminsfr = p->zmax - p->dz * (double)ceil((p->zmax - p->Zminsfr) / p->dz);
  if (p->Zminsfr < p->zmin) p->Zminsfr = p->zmin;
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

int sf21_read_halos(const char *path, long *nhalos, void **records) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  long nh = 0;
  if (fread(&nh, sizeof(long), 1, f) != 1 || nh < 0) { fclose(f); return 2; }
  void *h = malloc((size_t)16 * (size_t)(nh ? nh : 1));
  if (!h) { fclose(f); return 3; }
  if (fread(h, 16, (size_t)nh, f) != (size_t)nh) { free(h); fclose(f); return 2; }
  fclose(f);
  *nhalos = nh;
  *records = h;
  return 0;
}
