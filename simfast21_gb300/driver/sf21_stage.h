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
} sf21_stage_params;

/* Input_variables.c:16-141 restricted to the keys of the HII stage.
 * Returns 0, or nonzero if the file is missing or malformed. */
int sf21_read_params(const char *basedir, sf21_stage_params *p);

/* Raw float32 box of n values; 0 on success, nonzero on open/short read. */
int sf21_read_box(const char *path, float *buf, long n);
int sf21_write_box(const char *path, const float *buf, long n);

/* Halo branch source (get_HIIbubbles.c:229-253): reads the catalogue
 * (long nhalos, then {float Mass,x,y,z} per halo), deposits Rion(M, z) by
 * cloud-in-cell on the N_halo^3 grid in catalogue order (auxiliary.c:761-808)
 * and block-averages to N_smooth^3 (auxiliary.c:643-684).  The result is the
 * box before the *(dx_s/dx_h)^3*fesc of :258, i.e. SF21_SRC_RION input. */
int sf21_halo_rion_box(const char *path, double z, const sf21_stage_params *p, float *out);

#endif
