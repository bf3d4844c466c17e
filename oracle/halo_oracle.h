/*
 * CPU restatement of SimFast21's excursion-set halo finder (get_halos.c),
 * used ONLY as test infrastructure: the checker of the GPU halo finder and
 * its timed CPU baseline.  Nothing in the product library links or calls it.
 *
 * Parity pin: built against the same FFTW-API shim and GSL restatement, it
 * writes byte-identical catalogues to the reference's own get_halos.c
 * compiled unmodified from its sources (oracle/Makefile target _ref); the
 * fixtures under tests/golden/halos_*.npz were produced by that build.
 */
#ifndef SF21_HALO_ORACLE_H
#define SF21_HALO_ORACLE_H
#include <stdint.h>

#include "hii_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters after get_Simfast21_params (Input_variables.c:46-134). */
typedef struct {
  long N;         /* global_N_halo */
  double L;       /* global_L, Mpc/h (sim_length * hubble) */
  double hubble, omega_m, omega_b, omega_l, sig8, n_index;
  double delta_c, STa, STb, STc; /* critical_overdensity, Sheth-Tormen a, b, c */
  double Mmin, dlm;              /* halo_Mmin (Msun), halo_dlm */
  int use_sgrid;                 /* Use_subgrid */
  int nthreads;
} sf21o_hparams;

/* One mass of the excursion-set loop (get_halos.c:197-289). */
typedef struct {
  double M, R;   /* halo_mass (Msun), R (Mpc/h) */
  double dndm;   /* expected count in the box (:201) */
  double dcmz;   /* deltaCMZ = growth * deltaFilter(sigma(R), growth) (:205) */
  int active;    /* dndm > -log(0.9): the mass is searched (:203) */
} sf21o_hmass;

/* Scalars of auxiliary.c, restated in the same operation order. */
double sf21o_h_growth(const sf21o_hparams *p, double z);             /* getGrowth :262-266 */
double sf21o_h_sigma(const sf21o_hparams *p, double R);              /* sigma :415-424 */
double sf21o_h_mass_function(const sf21o_hparams *p, double z, double M); /* mass_function_ST :507-532 */
double sf21o_h_bias(const sf21o_hparams *p, double z, double sigmaM);    /* Bias :446-458 */

/* The mass list of the excursion-set loop for redshift z; writes up to cap
 * entries and returns the total count. */
int sf21o_halo_schedule(const sf21o_hparams *p, double z, sf21o_hmass *out, int cap);

/* The filtered, inverse-transformed field of mass index m of the schedule
 * (:211-229), N^3 floats unpadded.  Returns 0 on success. */
int sf21o_halo_field(const sf21o_hparams *p, double z, const float *delta_z0, int m, float *out);

/* One redshift of get_halos.c (:178-379).  delta_z0: the z = 0 linear
 * density box (N^3).  Writes up to cap records and returns the total number
 * of halos (-1 on failure).  rng: the taus generator's three state words,
 * read and written back (the reference keeps one generator for the whole
 * run, get_halos.c:70-71).  masks: NULL, or one candidate bit set per mass of
 * the schedule (bit t of word t/32 = cell t above the threshold; NULL entries
 * for inactive masses); when given, the candidates are taken from it
 * instead of the filtered fields and no transform runs.  counts (optional):
 * per schedule mass the number of halos found, then the cell-size cycle's. */
long sf21o_halo_find_z(const sf21o_hparams *p, double z, const float *delta_z0, sf21o_halo *out, long cap,
                       unsigned long rng[3], const uint32_t *const *masks, long *counts);

/* The generator's state after gsl_rng_set(r, seed) (get_halos.c:70-71). */
void sf21o_taus_seed(unsigned long seed, unsigned long rng[3]);

#ifdef __cplusplus
}
#endif
#endif
