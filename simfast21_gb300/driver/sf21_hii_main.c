/*
 * sf21_hii: drop-in replacement of SimFast21's get_HIIbubbles.x.
 *
 *   sf21_hii base_dir
 *
 * Same inputs and outputs as the reference stage (get_HIIbubbles.c:40-545):
 * reads base_dir/simfast21.ini, delta/deltanl_z*.dat and either
 * SFR/sfrd_z*.dat (use_SFR = T) or Halos/halonl_z*.dat.catalog (use_SFR = F);
 * writes Ionization/xHII_z*.dat (raw float32 N^3) and appends
 * Output_text_files/zsim.txt and Output_text_files/x_HI_N*_L*.dat.  The
 * per-redshift compute goes through libsf21hii.so (include/sf21_hii.h) on
 * one GPU; this file keeps the reference's host control flow, file names,
 * early stop and text outputs.
 *
 * Batched extension: an optional ini key `hii_param_sets = <file>` (ignored
 * by the reference's parser, Input_variables.c:38-108, like any unknown
 * key) names a text file with one "fesc bubble_Rmax[Mpc] bubble_Nbins" line
 * per extra parameter set.  Set k (k >= 1) writes its boxes and x_HI file
 * under Ionization/set<k>/ and Output_text_files/set<k>/; set 0 is the
 * ini's own fesc/bubble_Rmax/bubble_Nbins and writes where the reference
 * does.  All sets share one forward transform per redshift.
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

#include "sf21_hii.h"
#include "sf21_stage.h"

static void die(const char *msg) {
  printf("%s\n", msg);
  fflush(stdout);
  exit(1);
}

static void ensure_dir(const char *path, const char *what) {
  DIR *d = opendir(path);
  if (d) {
    closedir(d);
    return;
  }
  printf("Creating %s directory\n", what);
  if (mkdir(path, (S_IRWXU | S_IRGRP | S_IXGRP | S_IROTH | S_IXOTH)) != 0 && errno != EEXIST)
    die("Error creating directory!");
}

int main(int argc, char *argv[]) {
  char fname[1024];
  if (argc != 2) {
    printf("Generates boxes with ionization fraction for a range of redshifts\n");
    printf("usage: sf21_hii base_dir\n");
    printf("base_dir contains simfast21.ini and directory structure\n");
    return 1;
  }
  const char *base = argv[1];
  sf21_stage_params sp;
  if (sf21_read_params(base, &sp) != 0) die("\nThe parameter file simfast21.ini cannot be read. Exit...");

  /* parameter sets: the ini's own plus the optional batch file */
  sf21_hii_set sets[256];
  int nsets = 1;
  sets[0].fesc = sp.fesc;
  sets[0].Rmax = sp.bubble_Rmax;
  sets[0].Nbins = sp.bubble_Nbins;
  if (sp.param_sets_file[0]) {
    snprintf(fname, sizeof fname, "%s/%s", base, sp.param_sets_file);
    FILE *f = fopen(fname, "r");
    if (!f) die("Error opening hii_param_sets file");
    double fe, rm;
    int nb;
    while (nsets < 256 && fscanf(f, "%lf %lf %d", &fe, &rm, &nb) == 3) {
      rm *= sp.hubble; /* Mpc -> Mpc/h, Input_variables.c:123 */
      if (rm > sp.L / 2.) rm = sp.L / 2.;
      sets[nsets].fesc = fe;
      sets[nsets].Rmax = rm;
      sets[nsets].Nbins = nb;
      nsets++;
    }
    fclose(f);
  }

  snprintf(fname, sizeof fname, "%s/Ionization", base);
  ensure_dir(fname, "Ionization");
  snprintf(fname, sizeof fname, "%s/Output_text_files", base);
  ensure_dir(fname, "Output_text_files");
  for (int s = 1; s < nsets; s++) {
    snprintf(fname, sizeof fname, "%s/Ionization/set%d", base, s);
    ensure_dir(fname, "Ionization/set");
    snprintf(fname, sizeof fname, "%s/Output_text_files/set%d", base, s);
    ensure_dir(fname, "Output_text_files/set");
  }

  sf21_hii_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.N = sp.N_smooth;
  cfg.N_halo = sp.N_halo;
  cfg.L = sp.L;
  cfg.hubble = sp.hubble;
  cfg.device = 0;
  cfg.nsets = nsets;
  cfg.sets = sets;
  cfg.path = 0; /* tuned */
  sf21_hii_ctx *ctx = NULL;
  int rc = sf21_hii_create(&cfg, &ctx);
  if (rc != SF21_OK) {
    printf("sf21_hii_create failed (%d): %s\n", rc, sf21_hii_last_error(NULL));
    return 1;
  }

  const long N = sp.N_smooth, N3 = N * N * N;
  float *delta = malloc(sizeof(float) * N3);
  float *src = malloc(sizeof(float) * N3);
  float *xhii = malloc(sizeof(float) * N3 * nsets);
  double *neutral = calloc((size_t)nsets, sizeof(double));
  const double zmin = sp.zmin, zmax = sp.zmax, dz = sp.dz;
  const int nz = (int)((zmax - zmin) / dz + 2);
  double *xHI = calloc((size_t)nz * nsets, sizeof(double));
  if (!delta || !src || !xhii || !neutral || !xHI) die("Memory Problem...");
  for (int s = 0; s < nsets; s++) {
    double R[512];
    int nfft = 0;
    int nr = sf21_hii_radii(ctx, s, R, 512, &nfft);
    printf("Set %d: fesc %g, Rmax %g Mpc/h, %d radii (%d FFT branch)\n", s, sets[s].fesc, sets[s].Rmax, nr, nfft);
  }
  printf("Redshift cycle...\n");
  fflush(stdout);

  const double Lmpc = sp.L / sp.hubble;
  int iz = 0;
  double redshift;
  double gate = 0.; /* early stop on the ini's own set (:206) */
  for (redshift = zmin; redshift < (zmax + dz / 10) && (gate < sp.xHlim); redshift += dz) {
    printf("z = %f\n", redshift);
    fflush(stdout);
    snprintf(fname, sizeof fname, "%s/delta/deltanl_z%.3f_N%ld_L%.1f.dat", base, redshift, N, Lmpc);
    if (sf21_read_box(fname, delta, N3) != 0) die("\nError reading deltanl file... Check path or if the file exists...");
    if (sp.use_SFR) {
      snprintf(fname, sizeof fname, "%s/SFR/sfrd_z%.3f_N%ld_L%.1f.dat", base, redshift, N, Lmpc);
      if (sf21_read_box(fname, src, N3) != 0) die("\nError reading SFR file... Check path or if the file exists...");
      rc = sf21_hii_run_z(ctx, redshift, SF21_SRC_SFRD, delta, src, xhii, neutral);
    } else {
      /* halo branch: cloud-in-cell of Rion and smooth_box on the GPU (:229-259) */
      snprintf(fname, sizeof fname, "%s/Halos/halonl_z%.3f_N%ld_L%.1f.dat.catalog", base, redshift, sp.N_halo,
               Lmpc);
      long nh = 0;
      void *halos = NULL;
      if (sf21_read_halos(fname, &nh, &halos) != 0)
        die("\nError reading halo catalogue... Check path or if the file exists...");
      printf("Reading %ld halos...\n", nh);
      rc = sf21_hii_run_z_halos(ctx, redshift, delta, nh, halos, xhii, neutral);
      free(halos);
    }
    if (rc != SF21_OK) {
      printf("sf21_hii_run_z failed (%d): %s\n", rc, sf21_hii_last_error(ctx));
      return 1;
    }
    for (int s = 0; s < nsets; s++) {
      printf("neutral fraction=%lf%s\n", neutral[s], s ? " (set)" : "");
      xHI[(size_t)s * nz + iz] = neutral[s];
      if (s == 0)
        snprintf(fname, sizeof fname, "%s/Ionization/xHII_z%.3f_N%ld_L%.1f.dat", base, redshift, N, Lmpc);
      else
        snprintf(fname, sizeof fname, "%s/Ionization/set%d/xHII_z%.3f_N%ld_L%.1f.dat", base, s, redshift, N, Lmpc);
      if (sf21_write_box(fname, xhii + (size_t)s * N3, N3) != 0) {
        printf("Error opening file:%s\n", fname);
        return 1;
      }
    }
    fflush(stdout);
    gate = neutral[0];
    iz++;
  }

  /* remaining redshifts above the cutoff: all-neutral boxes (:494-513) */
  printf("Writing high redshift xHII boxes...\n");
  memset(xhii, 0, sizeof(float) * N3);
  while (redshift < (zmax + dz / 10)) {
    for (int s = 0; s < nsets; s++) {
      xHI[(size_t)s * nz + iz] = 1.0;
      if (s == 0)
        snprintf(fname, sizeof fname, "%s/Ionization/xHII_z%.3f_N%ld_L%.1f.dat", base, redshift, N, Lmpc);
      else
        snprintf(fname, sizeof fname, "%s/Ionization/set%d/xHII_z%.3f_N%ld_L%.1f.dat", base, s, redshift, N, Lmpc);
      if (sf21_write_box(fname, xhii, N3) != 0) {
        printf("Error opening file:%s\n", fname);
        return 1;
      }
    }
    iz++;
    redshift += dz;
  }

  /* text outputs (:515-528), appended, highest redshift first */
  snprintf(fname, sizeof fname, "%s/Output_text_files/zsim.txt", base);
  FILE *fid = fopen(fname, "a");
  if (!fid) {
    printf("Error opening file:%s\n", fname);
    return 1;
  }
  for (redshift = zmax; redshift > (zmin - dz / 10); redshift -= dz) fprintf(fid, "%f\n", redshift);
  fclose(fid);
  for (int s = 0; s < nsets; s++) {
    if (s == 0)
      snprintf(fname, sizeof fname, "%s/Output_text_files/x_HI_N%ld_L%.1f.dat", base, N, Lmpc);
    else
      snprintf(fname, sizeof fname, "%s/Output_text_files/set%d/x_HI_N%ld_L%.1f.dat", base, s, N, Lmpc);
    fid = fopen(fname, "a");
    if (!fid) {
      printf("Error opening file:%s\n", fname);
      return 1;
    }
    for (int i = iz - 1; i >= 0; i--) fprintf(fid, "%lf\n", xHI[(size_t)s * nz + i]);
    fclose(fid);
  }

  sf21_hii_destroy(ctx);
  free(delta);
  free(src);
  free(xhii);
  free(neutral);
  free(xHI);
  return 0;
}
