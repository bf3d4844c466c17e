/*
 * CPU restatement of the SimFast21 HII-bubble stage (get_HIIbubbles.c),
 * used ONLY as test infrastructure: the checker for the GPU library's
 * parity tests, the CPU baseline timed by bench.py, and smoke().
 * Nothing in the product library links or calls it.
 *
 * Parity pin: built against the same FFTW-API shim, this restatement gives
 * byte-identical xHII boxes to the reference's own get_HIIbubbles.c
 * compiled unmodified from its sources (oracle/Makefile target _ref); the
 * committed fixtures under tests/golden/ were produced by that build.
 */
#ifndef SF21_HII_ORACLE_H
#define SF21_HII_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters after get_Simfast21_params (Input_variables.c:119-134):
 * L and Rmax already multiplied by h and Rmax clamped to L/2. */
typedef struct {
  long N;        /* global_N_smooth */
  long N_halo;   /* global_N_halo (halo-catalogue branch only) */
  double L;      /* global_L, Mpc/h */
  double hubble; /* global_hubble */
  double Rmax;   /* global_bubble_Rmax, Mpc/h */
  int Nbins;     /* global_bubble_Nbins */
  double fesc;   /* global_fesc (the efficiency zeta) */
  int nthreads;  /* global_nthreads */
  int max_radii; /* 0 = the full radius schedule; n > 0 stops both loops
                    after the first n radii (a bounded CPU timing sample);
                    n < 0 runs the prologue, source conversion and
                    single-cell fill only (xhii = the uncapped fill) */
} sf21o_params;

/* Mirrors Halo_t (auxiliary.h:13-17). */
typedef struct {
  float Mass, x, y, z;
} sf21o_halo;

/* Radius list of the two bubble loops (get_HIIbubbles.c:192,298-299,397,
 * 402,461).  Writes up to cap radii into R (descending) and returns the
 * total count; *n_fft receives how many take the FFT branch (R >= 2 dx). */
int sf21o_radii(const sf21o_params *p, double *R, int cap, int *n_fft);

/* One redshift of the stage, SFR branch (use_SFR = T):
 * get_HIIbubbles.c:215-226, 262-275, 277-471.
 * delta, sfrd: N^3 float inputs (not modified).  xhii: N^3 output.
 * Optional outputs (NULL to skip): fresid, rec0 (Rrec box), ion0 (Rion box),
 * fill0 (single-cell fill before the radius loops).
 * *neutral receives the mean neutral fraction (:473-477).
 * Returns 0 on success, nonzero on allocation or plan failure. */
/* CPU-baseline timing sample: the front of one redshift (prologue, source
 * conversion, fill, forward transforms) and then the loop body of each
 * radius index ridx[0..n) on its own; wall seconds in *t_front and
 * t_radius[k]. */
int sf21o_time_radii(const sf21o_params *p, double z, const float *delta,
                     const float *sfrd, const int *ridx, int n,
                     double *t_front, double *t_radius);

int sf21o_run_z_sfr(const sf21o_params *p, double z, const float *delta,
                    const float *sfrd, float *xhii, float *fresid, float *rec0,
                    float *ion0, float *fill0, double *neutral);

/* Same, but the ionisation-rate box is given directly (already in Rion
 * units, i.e. what get_HIIbubbles.c holds in halo_map after :258 or :273). */
int sf21o_run_z_rion(const sf21o_params *p, double z, const float *delta,
                     const float *rion, float *xhii, float *fresid,
                     float *rec0, float *fill0, double *neutral);

/* Halo-catalogue source box (use_SFR = F): get_HIIbubbles.c:229-259, with
 * CIC (auxiliary.c:761-808) and smooth_box (auxiliary.c:643-684).
 * Writes the N^3 Rion box (times (dx_s/dx_h)^3 fesc) into out. */
int sf21o_halo_source(const sf21o_params *p, double z, long nhalos,
                      const sf21o_halo *halos, float *out);

/* The same box before the final *(dx_s/dx_h)^3*fesc of :258: CIC of
 * Rion(M, z) on the N_halo^3 grid, block-averaged to N^3 (:233-253). */
int sf21o_halo_smoothed(const sf21o_params *p, double z, long nhalos,
                        const sf21o_halo *halos, float *out);

/* SFRD box of the star-formation-rate stage (get_SFR.c:104-146): CIC of
 * sfr(M, z) = Rion/Qion on the N_halo^3 grid, block average to N^3, / dx_halo^3.
 * mean (may be NULL) receives the serial double average of :141-145. */
int sf21o_sfrd_box(const sf21o_params *p, double z, long nhalos,
                   const sf21o_halo *halos, float *out, double *mean);

/* Filtered fields at one radius exactly as the reference computes them
 * (:305-325): unnormalised c2r outputs of the filtered Rrec and Rion boxes. */
int sf21o_filtered(const sf21o_params *p, const float *rec0, const float *ion0,
                   double R, float *rec_R, float *ion_R);

/* Per-voxel physics helpers (user_functions.c:40-106), exposed for tests. */
double sf21o_Rion(float hmass, double z, const sf21o_params *p);
double sf21o_Rrec(float overdensity, double z, const sf21o_params *p);
double sf21o_G_H(double z);
double sf21o_XHI(double ratio);
double sf21o_Qion(double z);
double sf21o_W_filter(double x);

#ifdef __cplusplus
}
#endif
#endif
