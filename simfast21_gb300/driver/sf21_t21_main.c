/*
 * sf21_t21: drop-in for the reference's 21-cm stage t21.x on one GPU.
 *
 *   sf21_t21 base_dir
 *
 * Same inputs and outputs as t21.c:48-255: reads base_dir/simfast21.ini,
 * delta/deltanl_z*.dat, Ionization/xHII_z*.dat and, with use_Lya_xrays = T
 * above Zminsfr, x_c/xc_z*, Lya/xalpha_z* and xrays/TempX_z*; writes
 * deltaTb/deltaTb_z*.dat (float32, K) and appends
 * Output_text_files/t21_av_N*_L*.dat and TS_av_N*_L*.dat ("%f %.8E").
 * Redshifts from zmax down to zmin; an existing output box is skipped, as
 * the reference does.  The per-redshift work goes through sf21_t21_run_z.
 */
#define _POSIX_C_SOURCE 200809L
#include <dirent.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "sf21_hii.h"
#include "sf21_stage.h"

static int read_or_die(const char *fname, float *buf, long n) {
  if (sf21_read_box(fname, buf, n) != 0) {
    printf("Error opening file:%s\n", fname);
    exit(1);
  }
  return 0;
}

int main(int argc, char *argv[]) {
  char fname[1024];
  if (argc != 2) {
    printf("Usage : sf21_t21 base_dir\n");
    return 1;
  }
  const char *base = argv[1];
  sf21_stage_params sp;
  if (sf21_read_params(base, &sp) != 0) {
    printf("\nThe parameter file simfast21.ini cannot be open. Exit...\n");
    return 1;
  }
  if (sp.use_Lya_xrays == 0) printf("Lya and xray use set to false - assuming TS>>TCMB in t21 calculation.\n");
  snprintf(fname, sizeof fname, "%s/deltaTb", base);
  DIR *dir = opendir(fname);
  if (dir) {
    closedir(dir);
  } else {
    printf("Creating t21 directory\n");
    if (mkdir(fname, (S_IRWXU | S_IRGRP | S_IXGRP | S_IROTH | S_IXOTH)) != 0 && errno != EEXIST) {
      printf("Error creating directory!\n");
      return 1;
    }
  }
  const long N = sp.N_smooth, n3 = N * N * N;
  const double Lmpc = sp.L / sp.hubble;
  snprintf(fname, sizeof fname, "%s/Output_text_files/t21_av_N%ld_L%.1f.dat", base, N, Lmpc);
  FILE *fidtxt = fopen(fname, "a");
  snprintf(fname, sizeof fname, "%s/Output_text_files/TS_av_N%ld_L%.1f.dat", base, N, Lmpc);
  FILE *fidtxt2 = fidtxt ? fopen(fname, "a") : NULL;
  if (!fidtxt || !fidtxt2) {
    printf("\nError opening output %s file...\n", fname);
    return 1;
  }

  sf21_hii_set set = {1.0, sp.L / 4.0, 1};
  sf21_hii_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.N = N;
  cfg.N_halo = N;
  cfg.L = sp.L;
  cfg.hubble = sp.hubble;
  cfg.nsets = 1;
  cfg.sets = &set;
  cfg.kmax = 1;
  cfg.path = 1; /* no radius pipeline is used: skip the tuning */
  sf21_hii_ctx *ctx = NULL;
  if (sf21_hii_create(&cfg, &ctx) != SF21_OK) {
    printf("sf21_t21: %s\n", sf21_hii_last_error(NULL));
    return 1;
  }
  float *delta = malloc(sizeof(float) * n3), *xhii = malloc(sizeof(float) * n3), *tb = malloc(sizeof(float) * n3);
  float *xc = malloc(sizeof(float) * n3), *xa = malloc(sizeof(float) * n3), *tk = malloc(sizeof(float) * n3);
  if (!delta || !xhii || !tb || !xc || !xa || !tk) {
    printf("Problem...\n");
    return 1;
  }
  const sf21_t21_cosmo cosmo = {sp.omega_m, sp.omega_b, sp.omega_l, sp.vel_comp};
  const double zmin = sp.zmin, zmax = sp.zmax, dz = sp.dz;
  for (double z = zmax; z > (zmin - dz / 10); z -= dz) {
    printf("T21 - z = %f\n", z);
    fflush(stdout);
    snprintf(fname, sizeof fname, "%s/deltaTb/deltaTb_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
    FILE *fid = fopen(fname, "rb");
    if (fid) {
      printf("File:%s already exists - skipping this redshift...\n", fname);
      fclose(fid);
      continue;
    }
    const int spin = z > (sp.Zminsfr - dz / 10) && sp.use_Lya_xrays == 1;
    if (spin) {
      snprintf(fname, sizeof fname, "%s/x_c/xc_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
      read_or_die(fname, xc, n3);
      snprintf(fname, sizeof fname, "%s/Lya/xalpha_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
      read_or_die(fname, xa, n3);
      snprintf(fname, sizeof fname, "%s/xrays/TempX_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
      read_or_die(fname, tk, n3);
    }
    snprintf(fname, sizeof fname, "%s/delta/deltanl_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
    if (sf21_read_box(fname, delta, n3) != 0) {
      printf("Error reading deltanl file... Check path or if the file exists...");
      return 1;
    }
    snprintf(fname, sizeof fname, "%s/Ionization/xHII_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
    read_or_die(fname, xhii, n3);
    double mean_tb = 0., mean_ts = 0.;
    if (sf21_t21_run_z(ctx, &cosmo, z, delta, xhii, spin ? xc : NULL, spin ? xa : NULL, spin ? tk : NULL, tb,
                       &mean_tb, &mean_ts) != SF21_OK) {
      printf("sf21_t21: %s\n", sf21_hii_last_error(ctx));
      return 1;
    }
    snprintf(fname, sizeof fname, "%s/deltaTb/deltaTb_z%.3f_N%ld_L%.1f.dat", base, z, N, Lmpc);
    if (sf21_write_box(fname, tb, n3) != 0) {
      printf("Cannot open file:%s...\n", fname);
      return 1;
    }
    fprintf(fidtxt, "%f %.8E\n", z, mean_tb);
    if (spin) fprintf(fidtxt2, "%f %.8E\n", z, mean_ts);
  }
  fclose(fidtxt);
  fclose(fidtxt2);
  sf21_hii_destroy(ctx);
  free(delta);
  free(xhii);
  free(tb);
  free(xc);
  free(xa);
  free(tk);
  return 0;
}
