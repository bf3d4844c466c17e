/*
 * sf21_hii.h -- C-ABI of the GB300 HII-bubble filter bank (libsf21hii.so).
 *
 * Drop-in for the compute of SimFast21's get_HIIbubbles stage.  The stage's
 * executable keeps its I/O (simfast21.ini, delta/SFR/Halos boxes in,
 * Ionization/xHII boxes and text files out: get_HIIbubbles.c:63-96, 209-213,
 * 236-246, 263-267, 473-528); what it did in-process with FFTW plans and
 * OpenMP loops (get_HIIbubbles.c:98-194 and :215-471) is done behind these
 * entry points on one GPU.  Plain C types only; host buffers belong to the
 * caller, device buffers to the library (except in the *_device calls).
 *
 * Errors are returned as status codes (the reference printf()s and exit(1)s,
 * e.g. get_HIIbubbles.c:102-191); sf21_hii_last_error() gives the message.
 * A context is not thread-safe: one thread at a time per context.
 */
#ifndef SF21_HII_H
#define SF21_HII_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SF21_HII_ABI_VERSION 1

enum sf21_status {
  SF21_OK = 0,
  SF21_E_ARG = 1,         /* invalid argument (size, pointer, parameter)    */
  SF21_E_ALLOC = 2,       /* device or host allocation failed              */
  SF21_E_CUDA = 3,        /* CUDA runtime error                            */
  SF21_E_TIMEOUT = 4,     /* a bounded device wait expired                 */
  SF21_E_UNSUPPORTED = 5  /* configuration not supported (e.g. N not 2^k)  */
};

/* Source box kinds: what the caller passes as `src`.
 *  SF21_SRC_SFRD: SFRD box [Msun/(Mpc/h)^3/yr] (use_SFR = T), converted as
 *                 src*dx*dx*dx*Qion(z)*fesc   (get_HIIbubbles.c:272-274)
 *  SF21_SRC_RION: Rion box after CIC and smooth_box (use_SFR = F), converted
 *                 as src*pow(dx_s/dx_h,3)*fesc (get_HIIbubbles.c:257-259) */
enum sf21_src_kind { SF21_SRC_SFRD = 0, SF21_SRC_RION = 1 };

/* One efficiency / maximum-radius parameter set (the reference's fesc,
 * bubble_Rmax and bubble_Nbins after Input_variables.c:123-124). */
typedef struct {
  double fesc;   /* zeta (global_fesc)                                   */
  double Rmax;   /* global_bubble_Rmax in Mpc/h, already clamped to L/2  */
  int Nbins;     /* global_bubble_Nbins                                  */
} sf21_hii_set;

typedef struct {
  long N;            /* global_N_smooth: a power of two 16..1024, or a
                        product of 2, 3, 5 that 8 divides, 24..1280       */
  long N_halo;       /* global_N_halo (only for SF21_SRC_RION)             */
  double L;          /* global_L in Mpc/h (after the *h of Input_variables.c:121) */
  double hubble;     /* global_hubble                                       */
  int device;        /* CUDA device ordinal                                 */
  int nsets;         /* parameter sets sharing each forward transform (>=1) */
  const sf21_hii_set *sets;
  int kmax;          /* radii per spectrum read (0 = automatic: the
                        autotuner picks 8, 6 or 4; else fixed, <= 8)       */
  int path;          /* radius pipeline: 0 = tuned at create (times one batch
                        of each available one at each candidate batch size
                        and keeps the least time per radius; the timings
                        are cached per device, N and batch size in
                        $SF21_TUNE_CACHE or ~/.cache/simfast21_gb300/
                        tune.jsonl and reused, SF21_RETUNE=1 times again),
                        1 = three axis passes, 2 = plane passes on
                        thread-block clusters (N 64..512), 3 = three axis
                        passes with the ky pass TMA-pipelined and
                        persistent, 4 = ky and kx passes TMA-pipelined
                        (3 and 4: N 64..1024), 5-7 = the same over
                        column-block-major work boxes, 8 = column-block-
                        major c-axis pass + one persistent launch running
                        the ky and kx passes slab by slab through L2
                        (N 64..512) */
  int graph;         /* 0 = sf21_hii_run_z_device captures its per-redshift
                        schedule as a CUDA graph and replays it while z, the
                        kind, the buffers and the stream stay the same;
                        -1 = launch kernel by kernel */
} sf21_hii_config;

typedef struct sf21_hii_ctx sf21_hii_ctx;

/* Allocation, twiddle tables and per-set radius lists.
 * Replaces get_HIIbubbles.c:98-194 (fftwf_malloc of the boxes, the seven
 * FFTW_MEASURE plans, bfactor and the radius schedule of :298-461). */
int sf21_hii_create(const sf21_hii_config *cfg, sf21_hii_ctx **out);

/* Releases everything (get_HIIbubbles.c:530-541). */
int sf21_hii_destroy(sf21_hii_ctx *ctx);

/* Message of the last failing call on ctx (or of the last failed create
 * when ctx is NULL).  Replaces the printf() before exit(1). */
const char *sf21_hii_last_error(const sf21_hii_ctx *ctx);

/* One redshift, host buffers: the body of the redshift loop,
 * get_HIIbubbles.c:215-477 (prologue, source conversion, single-cell fill,
 * forward transforms, both radius loops, cap, neutral fraction).
 * delta, src: N^3 float (C order) as read from the deltanl and SFR/Rion files.
 * xhii: nsets * N^3 floats, set-major, each box in the byte layout the
 * reference writes to Ionization/xHII_*.dat (:485).
 * neutral: nsets doubles (may be NULL): the serial double mean of 1 - xHII
 * in the reference's order (:473-477). */
int sf21_hii_run_z(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta,
                   const float *src, float *xhii, double *neutral);

/* Same with device-resident buffers (no host copies); stream is a
 * cudaStream_t (NULL = the context's stream).  The call returns after
 * enqueueing; synchronise the stream before reading xhii. */
int sf21_hii_run_z_device(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta_dev,
                          const float *src_dev, float *xhii_dev, void *stream);

/* The plain form of one set, device buffers: the reference's per-radius
 * structure on the GPU, one radius per launch sequence -- filtered inverse
 * transform, centre mask, and for R >= 2 dx the FP32 FFT convolution of the
 * centres with the discrete sphere thresholded at 1/100 (:358-393), for
 * R < 2 dx the ball painting (:427-458).  Same outputs as sf21_hii_run_z for
 * that set (up to the reference's own FP32 convolution rounding).  Used as
 * the comparison baseline of the batched form. */
int sf21_hii_run_z_plain_device(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta_dev,
                                const float *src_dev, int set, float *xhii_dev, void *stream);

/* Halo-catalogue source (use_SFR = F): from the catalogue records
 * {float Mass, x, y, z} (Halo_t, auxiliary.h:13-17; positions in N_halo cell
 * units) builds on the GPU the box the reference holds in halo_map after
 * get_HIIbubbles.c:249-253 -- cloud-in-cell of Rion(M, z) on the N_halo^3 grid
 * in catalogue order and the block average to N_smoothed^3 -- bit-identical,
 * i.e. the SF21_SRC_RION input.  Replaces the serial loop :233-253. */
int sf21_hii_halo_source(sf21_hii_ctx *ctx, double z, long nhalos, const void *halos, float *rion_box);

/* Allocation-free form of sf21_hii_halo_source, for callers that may not
 * allocate device memory when they need the box (a fixed device-memory
 * budget after start-up, a host pool callback).  No reference counterpart:
 * the reference builds this box with its serial loop (:233-253).  No context;
 * device pointers: halos_dev holds nhalos records {float Mass, x, y, z},
 * rion_box_dev receives N_smoothed^3 floats, bit-identical with
 * sf21_hii_halo_source.  Its scratch is a fixed 16 MiB array in the
 * library's device image, so N_halo <= 128 and nhalos <= 16384; larger
 * requests return SF21_E_UNSUPPORTED before any GPU work (message in
 * sf21_hii_last_error(NULL)).  The first call in each CUDA context (the
 * current device's primary context) looks the array up
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is cached per context, so a call after cudaDeviceReset looks it
 * up again.  Calls that overlap on one device share the array and race:
 * serialise them.  Enqueues on stream (a cudaStream_t, NULL
 * = legacy default stream) and returns. */
int sf21_hii_halo_source_noalloc(double z, long N_halo, long N_smoothed, long nhalos, const void *halos_dev,
                                 float *rion_box_dev, void *stream);

/* One redshift of the halo branch end to end (source box + :215-477); the
 * source box stays on the GPU.  Same outputs as sf21_hii_run_z. */
int sf21_hii_run_z_halos(sf21_hii_ctx *ctx, double z, const float *delta, long nhalos, const void *halos,
                         float *xhii, double *neutral);

/* Power spectrum of a box of the context's size N^3 (cubic boxes only), the
 * reference's tools/power3d_f.c:124-194: window per axis (flag 0 top hat,
 * 1 Bartlett, 2 Welch, power3d_f.c:205-211), r2c transform, |F|^2 summed in
 * spherical bins round(|k|/dk), dk = 2 pi / (N dl), divided by the bin count,
 * the window's sum of squares and multiplied by dl^3.  Writes k[b] = b dk and
 * P[b] for b < min(nk, cap); returns nk = round(sqrt(3) N/2) + 1, or minus
 * an SF21_E_* code.  Host box / device box (enqueued on stream, then
 * synchronised). */
int sf21_hii_power_spectrum(sf21_hii_ctx *ctx, const float *box, int flag, double dl, double *k, double *P,
                            int cap);
int sf21_hii_power_spectrum_device(sf21_hii_ctx *ctx, const float *box_dev, int flag, double dl, double *k,
                                   double *P, int cap, void *stream);

/* 21-cm brightness temperature of one redshift, the reference's t21.c:114-255
 * on a context of the box's size: line-of-sight velocity gradient of the
 * density (FFT, k_axis^2/k^2 with axis = vel_comp: 1 first index, 2 second,
 * else third; inverse; times -dD/dt / L^3 / H(z) dx^3 / D(z); clamped to
 * [-0.5, 1]), spin-temperature factor (1 when xc, xalpha and tempx are NULL,
 * i.e. Lya/X-rays off or z below Zminsfr; else x/(1+x) (1 - Tcmb/TK), x = xc +
 * xalpha), T_b = 23 mK (1 + delta) t / (1 + dv) (0.7/h) (Omega_b h^2/0.02)
 * sqrt(0.15/Omega_m/h^2 (1+z)/10) (1 - xHII), in K, as float.  Host boxes of
 * N^3 floats; *tb_mean and *ts_mean (may be NULL) receive the box means of
 * T_b and of Tcmb/(1 - t) (the latter only with the spin boxes).  Growth,
 * dD/dt and H(z) are computed on the host as auxiliary.c:224-291 does. */
typedef struct {
  double omega_m, omega_b, omega_lambda; /* omega_matter, omega_baryon, omega_lambda */
  int vel_comp;                          /* Vel_comp */
} sf21_t21_cosmo;
int sf21_t21_run_z(sf21_hii_ctx *ctx, const sf21_t21_cosmo *cosmo, double z, const float *delta, const float *xhii,
                   const float *xc, const float *xalpha, const float *tempx, float *tb, double *tb_mean,
                   double *ts_mean);

/* Radius list of a set exactly as the reference iterates it (:192, 298-461):
 * writes up to cap radii (Mpc/h, descending), returns the count (or <0 on
 * error); *n_fft receives how many take the FFT branch (R >= 2 dx). */
int sf21_hii_radii(const sf21_hii_ctx *ctx, int set, double *R, int cap, int *n_fft);

/* Check hooks.  Prologue outputs of one redshift for set `set`: the
 * recombination-rate box (:222), the residual neutral fraction (:220-221)
 * and the single-cell fill (:281-288); any pointer may be NULL. */
int sf21_hii_prologue(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta,
                      const float *src, int set, float *rec0, float *fresid, float *fill0);

/* Filtered fields at radius index ridx of set `set`: rec_R and ion_R as the
 * reference's unnormalised c2r outputs hold them (:324-325). */
int sf21_hii_filtered(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta,
                      const float *src, int set, int ridx, float *rec_R, float *ion_R);

/* First-hit radius index per voxel of set `set` after the radius loops
 * (0xFF = never a bubble centre): the largest R at which the voxel passes
 * the centre test of :339-348 / :437-438. */
int sf21_hii_first_hit(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta,
                       const float *src, int set, uint8_t *rc);

/* Continuous ionisation criterion of set `set`: C(x) = max over the set's
 * FFT-branch radii (R >= 2 dx, :299) with rec_R(x) > 0 of ion_R(x) / rec_R(x)
 * (below 2 dx the top-hat's ringing takes rec_R through zero and the ratio is
 * ill-conditioned), the ratio the reference
 * thresholds at 1 (get_HIIbubbles.c:339-348, 437-438), and the radius index
 * of the maximum (argmax, 0xFF where no radius has rec_R > 0; C = 0 there).
 * No reference counterpart: the reference only tests ratio >= 1.  The
 * argmax stays in the context as the checkpoint of the next vjp call. */
int sf21_hii_criterion(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta,
                       const float *src, int set, float *C, uint8_t *argmax);
int sf21_hii_criterion_device(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta_dev,
                              const float *src_dev, int set, float *C_dev, uint8_t *argmax_dev,
                              void *stream);

/* Vector-Jacobian product of the criterion: given dC = dL/dC (N^3 floats),
 * dL/d delta, dL/d src (N^3 each, NULL to skip) and dL/d fesc (one double,
 * NULL to skip), for the same z, inputs and set as the preceding criterion
 * call on ctx (its argmax index is the only checkpoint; the filtered fields
 * are recomputed).  Away from argmax ties. No reference counterpart. */
int sf21_hii_vjp(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta, const float *src,
                 int set, const float *dC, float *ddelta, float *dsrc, double *dfesc);
int sf21_hii_vjp_device(sf21_hii_ctx *ctx, double z, int src_kind, const float *delta_dev,
                        const float *src_dev, int set, const float *dC_dev, float *ddelta_dev,
                        float *dsrc_dev, double *dfesc, void *stream);

/* Radius pipeline in use (1..8, see sf21_hii_config.path); ms_tuned[p-1]
 * receives the measured ms of one batch of pipeline p when it was tuned at
 * create (0 if not timed), for p <= cap. */
int sf21_hii_path(const sf21_hii_ctx *ctx, double *ms_tuned, int cap);

/* Radii per spectrum read (batch size K) in use: kmax when the config fixed
 * it, else the autotuner's choice among kmax (<= 8), 6 and 4 (least time per
 * radius together with the pipeline).  No reference counterpart. */
int sf21_hii_batch_radii(const sf21_hii_ctx *ctx);

/* Synchronises the context's stream and reports SF21_E_TIMEOUT if a bounded
 * device wait (TMA copy completion) expired since the last check. */
int sf21_hii_check(sf21_hii_ctx *ctx);

/* Polls per bounded device wait of the TMA-pipelined passes (pipelines 3, 4,
 * 6 and 7); 0 restores the default (2^26 polls, seconds).  A wait that runs
 * out makes its block record the error, wait for its own copies in flight
 * (always with the default bound) and return, so the context stays usable;
 * the next sf21_hii_check / host-buffer run reports SF21_E_TIMEOUT.  No
 * reference counterpart (the reference's FFTW calls have no device waits);
 * lowering it is how the timeout path is exercised without a real stall. */
int sf21_hii_set_wait_limit(sf21_hii_ctx *ctx, unsigned int polls);

/* Test hook: the n-th device allocation made by any of the library's
 * contexts after this call (n >= 1) fails with cudaErrorMemoryAllocation,
 * once; n = 0 disarms it.  The call that met the failure returns
 * SF21_E_ALLOC and frees what it had allocated (sf21_hii_create leaves
 * nothing behind).  No reference counterpart: the reference's allocation
 * checks (get_HIIbubbles.c:102-191) print and exit(1). */
int sf21_hii_inject_alloc_failure(long n);

/* Measurement hooks.  sf21_hii_profile(ctx, 1) starts recording CUDA events
 * around every kernel the context launches (on its launch stream) and clears
 * the totals; sf21_hii_profile_read() synchronises and returns the number of
 * kernel kinds K, filling ms[k] (summed device time) and launches[k] for
 * k < min(K, cap); sf21_hii_profile_name(k) names kind k.  No reference
 * counterpart (the reference has no timers, get_HIIbubbles.c:193-195). */
int sf21_hii_profile(sf21_hii_ctx *ctx, int enable);
int sf21_hii_profile_read(sf21_hii_ctx *ctx, double *ms, long *launches, int cap);
const char *sf21_hii_profile_name(int kind);

#ifdef __cplusplus
}
#endif
#endif
