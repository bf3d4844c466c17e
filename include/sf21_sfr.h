/*
 * sf21_sfr.h -- C ABI of the GPU star-formation-rate stage
 * (libsf21hii.so, sm_103a).
 *
 * Replaces the per-redshift body of the reference's get_SFR.c (the loop of
 * get_SFR.c:104-148): the halo catalogue's star-formation rates
 * sfr(M, z) = Rion(M, z) / Qion(z) (user_functions.c:71-75) deposited by
 * cloud-in-cell on the N_halo^3 grid (CIC, auxiliary.c:761-808, :119-121),
 * the block average to N_smoothed^3 (smooth_box, auxiliary.c:643-684, :123)
 * and the division by dx_halo^3 that turns the average into an SFR density in
 * Msun/(Mpc/h)^3/yr (:129-131).  The box is bit-identical with the
 * reference's serial loop: the CIC contributions are computed in parallel and
 * replayed per cell in the catalogue's order.  The per-redshift files
 * (SFR/sfrd_z*.dat and the Output_text_files/sfrd_av_* line) are written by
 * the drop-in driver sf21_get_SFR.
 *
 * Halo records: {float Mass, x, y, z} (Halo_t, auxiliary.h:13-17), positions
 * in N_halo cells.  Boxes: float32, C order (x slowest, z fastest).
 * Return codes are the SF21_* codes of sf21_hii.h.
 */
#ifndef SF21_SFR_H
#define SF21_SFR_H

#include "sf21_hii.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  long N_halo;      /* global_N_halo: the catalogue's grid                   */
  long N_smoothed;  /* global_N_smooth: the SFRD box side, <= N_halo          */
  double L;         /* box side in Mpc/h (sim_length * hubble)               */
  int device;       /* CUDA device ordinal                                   */
} sf21_sfr_config;

typedef struct sf21_sfr_ctx sf21_sfr_ctx;

int sf21_sfr_create(const sf21_sfr_config *cfg, sf21_sfr_ctx **out);
void sf21_sfr_destroy(sf21_sfr_ctx *ctx);
/* Message of the last failure on ctx, or of the last failed create (NULL ctx). */
const char *sf21_sfr_last_error(const sf21_sfr_ctx *ctx);

/* One redshift from host buffers: nhalos records in, the N_smoothed^3 SFRD box
 * out.  sfrd_mean (may be NULL) receives the box average as get_SFR.c:141-146
 * computes it (a serial double sum in index order, divided by N_smoothed^3). */
int sf21_sfr_box(sf21_sfr_ctx *ctx, double z, long nhalos, const void *halos, float *sfrd, double *sfrd_mean);

/* The same on device buffers, enqueued on stream (NULL: the legacy default
 * stream); returns without waiting for the result. */
int sf21_sfr_box_device(sf21_sfr_ctx *ctx, double z, long nhalos, const void *halos_dev, float *sfrd_dev,
                        void *stream);

#ifdef __cplusplus
}
#endif
#endif
