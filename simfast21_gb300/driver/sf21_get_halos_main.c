/*
 * sf21_get_halos: drop-in for the reference's halo finder get_halos.x on
 * one GPU.
 *
 *   sf21_get_halos work_dir
 *
 * Same inputs and outputs as get_halos.c:31-394: reads work_dir/simfast21.ini
 * and delta/delta_z0_N<N_halo>_L<L/h>.dat (the z = 0 linear density), and for
 * each redshift from zmax down to zmin writes
 * Halos/halo_z<z>_N<N_halo>_L<L/h>.dat.catalog: an int64 halo count, then the
 * {float Mass, x, y, z} records (Halo_t) in the reference's order.  A
 * catalogue that already exists is skipped, as the reference does (:174-177);
 * the subgrid generator runs on across the redshifts of one invocation, as
 * the reference's single gsl_rng does (:70-71).  The per-redshift work goes
 * through sf21_halo_find_z (N_halo: a power of two in [16, 1024], or a
 * product of 2, 3 and 5 that 8 divides in [24, 1280]).
 */
#define _POSIX_C_SOURCE 200809L
#include <dirent.h>
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "sf21_halos.h"
#include "sf21_stage.h"

int main(int argc, char **argv) {
  char fname[1024];
  if (argc != 2) {
    printf("Generates Halo catalogs for a range of redshifts\n");
    printf("Usage: sf21_get_halos work_dir\n");
    printf("work_dir - directory containing simfast21.ini \n");
    return 1;
  }
  const char *base = argv[1];
  sf21_stage_params sp;
  if (sf21_read_params(base, &sp) != 0) {
    printf("\nThe parameter file simfast21.ini cannot be open. Exit...\n");
    return 1;
  }
  sf21_halo_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.N_halo = sp.N_halo;
  cfg.L = sp.L;
  cfg.hubble = sp.hubble;
  cfg.omega_m = sp.omega_m;
  cfg.omega_b = sp.omega_b;
  cfg.omega_lambda = sp.omega_l;
  cfg.sigma8 = sp.sigma8;
  cfg.n_index = sp.n_index;
  cfg.delta_c = sp.delta_c;
  cfg.STa = sp.STa;
  cfg.STb = sp.STb;
  cfg.STc = sp.STc;
  cfg.halo_Mmin = sp.halo_Mmin;
  cfg.halo_dlm = sp.halo_dlm;
  cfg.use_subgrid = sp.use_sgrid;
  cfg.device = 0;
  const long N = sp.N_halo, n3 = N * N * N;
  const double Lmpc = sp.L / sp.hubble;

  sf21_halo_ctx *ctx = NULL;
  if (sf21_halo_create(&cfg, &ctx) != SF21_OK) {
    printf("sf21_get_halos: %s\n", sf21_halo_last_error(NULL));
    return 1;
  }
  float *delta = malloc(sizeof(float) * (size_t)n3);
  if (!delta) {
    printf("Memory problem - map_in_f...\n");
    return 1;
  }
  printf("Reading dark matter density box\n");
  fflush(stdout);
  snprintf(fname, sizeof fname, "%s/delta/delta_z0_N%ld_L%.1f.dat", base, N, Lmpc);
  if (sf21_read_box(fname, delta, n3) != 0) {
    printf("Error reading delta density file %s - check if the file exists...\n", fname);
    return 1;
  }
  if (sf21_halo_set_density(ctx, delta) != SF21_OK) {
    printf("sf21_get_halos: %s\n", sf21_halo_last_error(ctx));
    return 1;
  }
  free(delta);
  snprintf(fname, sizeof fname, "%s/Halos", base);
  DIR *dir = opendir(fname);
  if (dir) {
    closedir(dir);
  } else {
    printf("Creating Halo directory\n");
    if (mkdir(fname, (S_IRWXU | S_IRGRP | S_IXGRP | S_IROTH | S_IXOTH)) != 0 && errno != EEXIST) {
      printf("Error creating directory!\n");
      return 1;
    }
  }
  const double rho_m = sp.omega_m * 2.775e11 / sp.hubble; /* Input_variables.c:119 */
  const double dx = sp.L / N;
  const double mass_dx = rho_m * pow(dx, 3) * pow(10.0, sp.halo_dlm);
  printf("Mininum halo mass for excursion set formalism: %E\n", mass_dx);
  if (mass_dx > sp.halo_Mmin && sp.use_sgrid == 0)
    printf("Warning - minimum mass for box resolution is larger than halo_Mmin: you need to use subgrid to achieve "
           "that minimum mass.\n");
  printf("Redshift cycle...\n");
  fflush(stdout);

  enum { CHUNK = 1 << 20 };
  sf21_halo_rec *buf = malloc(sizeof(sf21_halo_rec) * CHUNK);
  sf21_halo_mass *ms = malloc(sizeof(sf21_halo_mass) * 4096);
  long *counts = malloc(sizeof(long) * 4100);
  if (!buf || !ms || !counts) {
    printf("Memory problem - halo_cat\n");
    return 1;
  }
  for (double z = sp.zmax; z > (sp.zmin - sp.dz / 10); z -= sp.dz) {
    printf("\n+++++++++++++++++++++++++++ z = %f +++++++++++++++++++++++++++++++\n", z);
    fflush(stdout);
    snprintf(fname, sizeof fname, "%s/Halos/halo_z%.3f_N%ld_L%.1f.dat.catalog", base, z, N, Lmpc);
    FILE *fid = fopen(fname, "rb");
    if (fid) {
      printf("File:%s already exists - skipping this redshift\n", fname);
      fclose(fid);
      continue;
    }
    long nh = 0;
    if (sf21_halo_find_z(ctx, z, &nh) != SF21_OK) {
      printf("sf21_get_halos: %s\n", sf21_halo_last_error(ctx));
      return 1;
    }
    const int nm = sf21_halo_schedule(&cfg, z, ms, 4096);
    const int nc = sf21_halo_counts(ctx, counts, 4100);
    long n_exc = 0;
    for (int m = 0; m < nm && m < nc; m++)
      if (ms[m].active) {
        printf("Number of halos for M=%E: %ld\n", ms[m].M, counts[m]);
        n_exc += counts[m];
      }
    printf("\n--------------- Number of halos without subgrid: %ld -----------------------\n\n", n_exc);
    if (nm + 1 < nc && rho_m * pow(dx, 3) >= sp.halo_Mmin)
      printf("Number of halos found in cell size cycle: %ld\n", counts[nm]);
    if (sp.use_sgrid == 1)
      printf("----------------------------- Total number of halos including subgrid: %ld ---------------------- \n\n",
             nh);
    fid = fopen(fname, "wb");
    if (!fid) {
      printf("\n Catalog file error\n");
      return 1;
    }
    if (fwrite(&nh, sizeof(long), 1, fid) != 1) {
      printf("\n Catalog file error\n");
      return 1;
    }
    for (long first = 0; first < nh; first += CHUNK) {
      const long k = nh - first < CHUNK ? nh - first : CHUNK;
      if (sf21_halo_fetch(ctx, buf, first, k) != SF21_OK) {
        printf("sf21_get_halos: %s\n", sf21_halo_last_error(ctx));
        return 1;
      }
      if (fwrite(buf, sizeof(sf21_halo_rec), (size_t)k, fid) != (size_t)k) {
        printf("\n Catalog file error\n");
        return 1;
      }
    }
    fclose(fid);
  }
  free(buf);
  free(ms);
  free(counts);
  sf21_halo_destroy(ctx);
  return 0;
}
