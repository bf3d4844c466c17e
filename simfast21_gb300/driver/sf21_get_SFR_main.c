/*
 * sf21_get_SFR: drop-in for the reference's star-formation-rate stage
 * get_SFR.x on one GPU.
 *
 *   sf21_get_SFR work_dir
 *
 * Same inputs and outputs as get_SFR.c:28-153: reads work_dir/simfast21.ini
 * and, for each redshift from zmax down to zmin (Zminsfr when only
 * Lya/X-rays need the boxes, :52-55), Halos/halonl_z<z>_N<N_halo>_L<L>.dat.catalog;
 * writes SFR/sfrd_z<z>_N<N_smoothed>_L<L>.dat (float32, Msun/(Mpc/h)^3/yr)
 * and appends "z mean" to Output_text_files/sfrd_av_N<N_smoothed>_L<L>.dat
 * (:88-92, :146).  The box comes from sf21_sfr_box (CIC of sfr(M, z) +
 * smooth_box + / dx_halo^3 on the GPU, bit-identical with the reference).
 */
#define _POSIX_C_SOURCE 200809L
#include <dirent.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "sf21_sfr.h"
#include "sf21_stage.h"

static int ensure_dir(const char *path, const char *msg) {
  DIR *dir = opendir(path);
  if (dir) {
    closedir(dir);
    return 0;
  }
  printf("%s", msg);
  if (mkdir(path, (S_IRWXU | S_IRGRP | S_IXGRP | S_IROTH | S_IXOTH)) != 0 && errno != EEXIST) {
    printf("Error creating directory!\n");
    return 1;
  }
  return 0;
}

int main(int argc, char **argv) {
  char fname[1024];
  if (argc != 2) {
    printf("Generates SFRD using nonlinear halo catalogue.\n");
    printf("usage: get_SFR base_dir\n");
    printf("base_dir contains simfast21.ini\n");
    return 1;
  }
  const char *base = argv[1];
  sf21_stage_params sp;
  if (sf21_read_params(base, &sp) != 0) {
    printf("\nThe parameter file simfast21.ini cannot be open. Exit...\n");
    return 1;
  }
  if (sp.use_Lya_xrays == 0 && sp.use_SFR == 0) {
    printf("SFR, Lya and xray use set to false - no need to calculate SFR\n");
    return 0;
  }
  const double zmin = sp.use_SFR == 1 ? sp.zmin : sp.Zminsfr, zmax = sp.zmax, dz = sp.dz;
  const double Lmpc = sp.L / sp.hubble;
  printf("\nCalculating SFRD between z=%f and z=%f with step %f\n", zmin, zmax, dz);
  printf("Using %d threads\n", sp.nthreads);

  snprintf(fname, sizeof fname, "%s/SFR", base);
  if (ensure_dir(fname, "Creating SFR directory\n")) return 1;
  sf21_sfr_config cfg = {sp.N_halo, sp.N_smooth, sp.L, 0};
  sf21_sfr_ctx *ctx = NULL;
  if (sf21_sfr_create(&cfg, &ctx) != SF21_OK) {
    printf("sf21_get_SFR: %s\n", sf21_sfr_last_error(NULL));
    return 1;
  }
  const long n3 = sp.N_smooth * sp.N_smooth * sp.N_smooth;
  float *box = malloc(sizeof(float) * (size_t)n3);
  if (!box) {
    printf("Problem...\n");
    return 1;
  }
  snprintf(fname, sizeof fname, "%s/Output_text_files", base);
  if (ensure_dir(fname, "Creating Output_text_files directory\n")) return 1;
  snprintf(fname, sizeof fname, "%s/Output_text_files/sfrd_av_N%ld_L%.1f.dat", base, sp.N_smooth, Lmpc);
  FILE *fid_sa = fopen(fname, "a");
  if (!fid_sa) {
    printf("\nError opening output %s file...\n", fname);
    return 1;
  }
  for (double z = zmax; z > (zmin - dz / 10); z -= dz) {
    snprintf(fname, sizeof fname, "%s/Halos/halonl_z%.3f_N%ld_L%.1f.dat.catalog", base, z, sp.N_halo, Lmpc);
    long nhalos = 0;
    void *halos = NULL;
    if (sf21_read_halos(fname, &nhalos, &halos) != 0) {
      printf("\nError reading %s file... Check path or if the file exists...", fname);
      return 1;
    }
    printf("Redshift: %f. Reading %ld halos...\n", z, nhalos);
    fflush(stdout);
    double mean = 0.0;
    if (sf21_sfr_box(ctx, z, nhalos, halos, box, &mean) != SF21_OK) {
      printf("sf21_get_SFR: %s\n", sf21_sfr_last_error(ctx));
      return 1;
    }
    free(halos);
    printf("Writing SFRD file...\n");
    snprintf(fname, sizeof fname, "%s/SFR/sfrd_z%.3f_N%ld_L%.1f.dat", base, z, sp.N_smooth, Lmpc);
    if (sf21_write_box(fname, box, n3) != 0) {
      printf("\nError opening %s file...\n", fname);
      return 1;
    }
    fprintf(fid_sa, "%f %.8E\n", z, mean);
  }
  fclose(fid_sa);
  free(box);
  sf21_sfr_destroy(ctx);
  return 0;
}
