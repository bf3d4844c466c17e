/*
 * Host side of the HII stage for the sf21_hii driver: simfast21.ini with
 * the reference's parsing rules and unit conversions, raw box I/O, and the
 * halo-catalogue source box (cloud-in-cell + block average on the host).
 */
#ifndef SF21_STAGE_H
#define SF21_STAGE_H

typedef struct {
  int nthreads;
  double zmin, zmax, dz;   /* zmin re-snapped as Input_variables.c:133 */
  double L;                /* Mpc/h (Input_variables.c:121) */
  double hubble;
  long N_halo, N_smooth;
  double fesc, xHlim;
  double bubble_Rmax;      /* Mpc/h, clamped to L/2 (Input_variables.c:123-124) */
  int bubble_Nbins;
  int use_SFR;
  char param_sets_file[512]; /* optional key hii_param_sets (batched sets) */
  /* keys of the 21-cm stage (t21.c) */
  double omega_m, omega_b, omega_l; /* omega_matter, omega_baryon, omega_lambda */
  int vel_comp;                     /* Vel_comp */
  int use_Lya_xrays;                /* use_Lya_xrays (default F, Input_variables.c:35) */
  double Zminsfr;                   /* re-snapped as Input_variables.c:134-137 */
  /* keys of the halo finder (get_halos.c) */
  double sigma8, n_index;           /* sigma8, spectral_index */
  double delta_c, STa, STb, STc;    /* critical_overdensity, STa, STb, STc */
  int use_sgrid;                    /* Use_subgrid (T -> 1, anything else 0) */
  double halo_Mmin, halo_dlm;       /* halo_Mmin, halo_dlm */
} sf21_stage_params;

/* Input_variables.c:16-141 restricted to the keys of the HII, 21-cm and halo stages.
 * Returns 0, or nonzero if the file is missing or malformed. */
int sf21_read_params(const char *basedir, sf21_stage_params *p);

/* Raw float32 box of n values; 0 on success, nonzero on open/short read. */
int sf21_read_box(const char *path, float *buf, long n);
int sf21_write_box(const char *path, const float *buf, long n);

/* Halo catalogue (Halos/halonl_z*.dat.catalog, output_files.txt:33-41):
 * long nhalos, then nhalos records {float Mass, x, y, z} (Halo_t,
 * auxiliary.h:13-17).  *records is malloc'ed (16 B per halo).  The source
 * box itself is built on the GPU by sf21_hii_run_z_halos. */
int sf21_read_halos(const char *path, long *nhalos, void **records);

#endif
