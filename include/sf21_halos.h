/*
 * sf21_halos.h -- C ABI of the GPU excursion-set halo finder
 * (libsf21hii.so, sm_103a).
 *
 * Replaces the per-redshift body of the reference's get_halos.c (the loop of
 * get_halos.c:178-379): for each mass from L/2 down to the cell mass, a
 * k-space top-hat filter of the z = 0 density spectrum and an inverse
 * transform (:211-229), the threshold against the Sheth-Tormen barrier and
 * the overlap test in scan order (:236-282), then the cell-size cycle
 * (:293-321) and the subgrid Poisson cycle (:326-371).  The catalogue has the
 * reference's records and order (Halo_t, auxiliary.h:13-17); the file layout
 * (an int64 count, then the records, :184-185, :272, :375-376) is written by
 * the drop-in driver sf21_get_halos.
 *
 * Boxes: N_halo^3 float32, C order (x slowest, z fastest).  N_halo a power of
 * two from 16 to 1024 (register transforms), or a product of 2, 3 and 5 with
 * 8 | N_halo from 24 to 1280 such as the reference's default 1200
 * (shared-memory transforms).
 * Return codes are the SF21_* codes of sf21_hii.h.
 */
#ifndef SF21_HALOS_H
#define SF21_HALOS_H

#include <stdint.h>

#include "sf21_hii.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters as get_Simfast21_params derives them (Input_variables.c:46-134). */
typedef struct {
  long N_halo;         /* cells per side (global_N_halo)                        */
  double L;            /* box side in Mpc/h (sim_length * hubble)               */
  double hubble;       /* h                                                      */
  double omega_m, omega_b, omega_lambda;
  double sigma8;       /* sigma8 (global_sig8_new)                               */
  double n_index;      /* spectral_index                                        */
  double delta_c;      /* critical_overdensity                                  */
  double STa, STb, STc;/* Sheth-Tormen barrier parameters                       */
  double halo_Mmin;    /* Msun                                                   */
  double halo_dlm;     /* log10 mass step                                        */
  int use_subgrid;     /* Use_subgrid = T                                        */
  int device;          /* CUDA device ordinal                                    */
} sf21_halo_config;

/* One catalogue record (Halo_t, auxiliary.h:13-17). */
typedef struct {
  float Mass, x, y, z;
} sf21_halo_rec;

/* One mass of the excursion-set loop (get_halos.c:197-289). */
typedef struct {
  double M;     /* halo mass, Msun                                           */
  double R;     /* radius, Mpc/h                                             */
  double dndm;  /* expected number in the box (:201)                         */
  double dcmz;  /* barrier deltaCMZ (:204-205); 0 when inactive               */
  int active;   /* dndm > -log(0.9): the mass is searched (:203)             */
  int nc;       /* sphere half-width in cells, (long)(R/dx), at least 1      */
} sf21_halo_mass;

typedef struct sf21_halo_ctx sf21_halo_ctx;

/* Host-side schedule of the excursion-set masses for redshift z; writes up
 * to cap entries and returns the total count, or minus an SF21_E code.
 * Replaces the scalar work of get_halos.c:195-206, 284-287 (sigma, mass
 * function, barrier: auxiliary.c:377-441, 507-532, growth :262-266). */
int sf21_halo_schedule(const sf21_halo_config *cfg, double z, sf21_halo_mass *out, int cap);

int sf21_halo_create(const sf21_halo_config *cfg, sf21_halo_ctx **out);
void sf21_halo_destroy(sf21_halo_ctx *ctx);
/* Message of the last failure on ctx, or of the last failed create (NULL ctx). */
const char *sf21_halo_last_error(const sf21_halo_ctx *ctx);

/* The z = 0 linear density box (get_halos.c:127-138): host / device pointer.
 * Its forward transform is taken once and reused by every redshift. */
int sf21_halo_set_density(sf21_halo_ctx *ctx, const float *delta_z0);
int sf21_halo_set_density_device(sf21_halo_ctx *ctx, const float *delta_z0_dev, void *stream);

/* One redshift (get_halos.c:178-379).  The catalogue stays on the device
 * until the next call; *nhalos receives its length.  The subgrid cycle
 * continues the context's generator (one generator for the whole run, as
 * get_halos.c:70-71). */
int sf21_halo_find_z(sf21_halo_ctx *ctx, double z, long *nhalos);

/* Copy records [first, first + count) of the last catalogue to host memory. */
int sf21_halo_fetch(sf21_halo_ctx *ctx, sf21_halo_rec *out, long first, long count);
/* Device pointer of the last catalogue (valid until the next find_z). */
const sf21_halo_rec *sf21_halo_catalogue_device(const sf21_halo_ctx *ctx);

/* Halos per schedule mass of the last find_z (the reference's "Number of
 * halos for M=..." lines, :281), then the cell-size cycle's (:320) and the
 * subgrid's (:372 minus the rest); returns the count written (schedule
 * length + 2) or minus an SF21_E code. */
int sf21_halo_counts(const sf21_halo_ctx *ctx, long *counts, int cap);

/* The subgrid generator's state: three 32-bit words of the taus generator
 * (gsl_rng_taus).  get: copies it out; set: replaces it (NULL = seed 0, the
 * reference's gsl_rng_set(rpoisson, 0)). */
int sf21_halo_rng_get(const sf21_halo_ctx *ctx, uint32_t state[3]);
int sf21_halo_rng_set(sf21_halo_ctx *ctx, const uint32_t state[3]);

/* Test hooks.  Candidate bit set (bit t of word t/32 = cell above the
 * barrier) of schedule mass m from the last find_z (N^3/32 words), or its
 * filtered field (N^3 floats, recomputed). */
int sf21_halo_candidates(const sf21_halo_ctx *ctx, int m, uint32_t *bits);
int sf21_halo_field(sf21_halo_ctx *ctx, double z, int m, float *out);

#ifdef __cplusplus
}
#endif
#endif
