// Internal launch API between the C-ABI layer (hii_api.cu) and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "prologue_fast.h"
#include "sf21_device.cuh"
#include "softdouble.h"

namespace sf21 {

// Device allocations of the library's contexts (HII, halo finder, SFR
// stage) go through dev_malloc, where sf21_hii_inject_alloc_failure can make
// a chosen one fail with cudaErrorMemoryAllocation (a test hook; off unless
// armed).
cudaError_t dev_malloc(void** p, size_t bytes);
template <class T>
inline cudaError_t dev_malloc(T** p, size_t bytes) {
  return dev_malloc(reinterpret_cast<void**>(p), bytes);
}

// Per-redshift scalars of the prologue, as IEEE double bit patterns computed
// on the host exactly as the reference evaluates them.
struct PrologueArgs {
  uint64_t one_plus_z_cubed;  // pow(1+z, 3.0)                 (:220)
  uint64_t g_h;               // G_H(z)                         (:220)
  uint64_t rec1;              // 1e-24*r1*pow(1+z, r4)          (user_functions.c:59)
  uint64_t dvv;               // pow(L*CM/N/h/(1+z), 3.0)       (user_functions.c:62)
  uint64_t c_resid;           // 1.881e-7                       (:220)
  uint64_t r2, r3;            // Rrec fit constants             (user_functions.c:54-55)
  uint64_t v_norm;            // 1e45                           (user_functions.c:38)
  uint64_t src_mul[6];        // source multipliers before zeta (:273 or :258)
  int n_src_mul;
  sd_divc r2c, v_normc;       // r2 and v_norm as prepared divisors (sd_div_c)
  RrecFast rf;                // fast-path constants (prologue_fast.h): Rrec,
  ProdFast pf_resid, pf_src;  // the residual-fraction product, the source product
};

cudaError_t fft_setup(int N);
// c-axis forward of the packed box (imag part times *alpha), in -> out
cudaError_t launch_fwd_rows(int N, const float2* in, float2* out, const float* alpha, const float2* tw,
                            cudaStream_t st);
// c-axis inverse in place, no filter
cudaError_t launch_inv_rows_plain(int N, float2* box, const float2* tw, cudaStream_t st);
// c-axis inverse with the top-hat filter of the batch's K radii: spec -> bt.r[k].work
cudaError_t launch_inv_rows_filter(int N, const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st);
// strided axis (1 = b, 0 = a) in place, of `box` (nbox = 1) or of the batch's work boxes
cudaError_t launch_cols(int N, float2* box, const Batch& bt, int nbox, int axis, bool inverse, const float2* tw,
                        cudaStream_t st);
// a-axis inverse of the batch's work boxes + centre test + first-hit update
cudaError_t launch_cols_a_test(int N, const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                               cudaStream_t st);

cudaError_t launch_prologue(long n3, const float* delta, const float* src, const PrologueArgs& pa,
                            float* rec0, float* fres, float2* packed, float* partials, int nblocks,
                            cudaStream_t st);
cudaError_t launch_alpha(const float* partials, int nblocks, float* alpha, cudaStream_t st);
int prologue_blocks(long n3);

// Dilation of the first-hit radius field and the final xHII box of one set
// (kernels_dt.cu): three max-plus passes (a: rc -> i1, b: i1 -> i2,
// c: i2 -> xhii); the last one also applies the single-cell fill and the cap.
// finish_prep, once per redshift: source chain before zeta (double bits) and
// 1 - fresid rounded down / to nearest per voxel.
cudaError_t dt_setup(int N);
cudaError_t launch_dt_pa(int N, const uint8_t* rc, const int* nmax, int* i1, cudaStream_t st);
cudaError_t launch_dt_pb(int N, const int* i1, int* i2, cudaStream_t st);
cudaError_t launch_dt_pc_finish(int N, const int* i2, uint64_t zeta, const uint64_t* chain, const float* rec0,
                                const float2* om, float* xhii, cudaStream_t st);
cudaError_t launch_finish_prep(long n3, const float* src, const float* fres, const PrologueArgs& pa, uint64_t* chain,
                               float2* om, cudaStream_t st);
cudaError_t launch_fill0(long n3, uint64_t zeta, const float* src, const float* rec0,
                         const PrologueArgs& pa, float* fill, cudaStream_t st);

// Plane pass on thread-block clusters (kernels_plane.cu): filter + kz + ky of
// whole kx planes for the batch's K radii, into the work boxes.
bool plane_supported(int N);
cudaError_t plane_setup(int N);
int plane_max_active_clusters(int N);
cudaError_t launch_plane_filter(int N, const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st);

// TMA-pipelined persistent strided passes (kernels_pipe.cu).  The K work
// boxes must be consecutive N^3 slices of one allocation starting at work0.
struct PipeMaps {
  CUtensorMap b_rows;     // tiles of rows along b (ky pass), natural layout
  CUtensorMap a_rows;     // tiles of rows along a (kx pass), natural layout
  CUtensorMap b_rows_cb;  // the same over the column-block-major layout
  CUtensorMap a_rows_cb;
};
bool pipe_supported(int N);
cudaError_t pipe_setup(int N);
cudaError_t pipe_make_maps(int N, PipeMaps* pm, int K, void* work_base);
// mode 0: ky inverse pass in place over the batch's boxes; mode 1: kx inverse
// pass + centre test + first-hit update.  layout 0: natural work boxes,
// 1: column-block major (kernels_cb.cu).  nsm = persistent CTAs.
// spin_limit: polls per bounded mbarrier wait (0 = the default, 2^26).
cudaError_t launch_pipe(int N, int mode, int layout, const PipeMaps& pm, const Batch& bt, float2* work0,
                        uint8_t* rc, const float* alpha, const float2* tw, int* err, int nsm, cudaStream_t st,
                        uint32_t spin_limit = 0);

// Radius pipeline over column-block-major work boxes (kernels_cb.cu):
// c-axis filter pass, in-place b-axis pass, a-axis pass + centre test.
cudaError_t cb_setup(int N);
cudaError_t launch_rows_filter_cb(int N, const float2* spec, const Batch& bt, const float2* tw, cudaStream_t st);
cudaError_t launch_cols_b_cb(int N, const Batch& bt, const float2* tw, cudaStream_t st);
cudaError_t launch_cols_a_test_cb(int N, const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw, int nsm,
                                  cudaStream_t st);

// b- and a-axis passes of a batch in one persistent launch through L2
// (kernels_fused.cu, radius pipeline 8; column-block-major work boxes).
// ctl: fused_ctl_ints(N) ints of device memory (zeroed by the launch).
bool fused_supported(int N);
size_t fused_ctl_ints(int N);
cudaError_t fused_setup(int N);
// rc32: 32-bit first-hit box (all bits set = never), folded into the byte box by launch_rc32_to_rc
cudaError_t launch_cols_ba_fused(int N, const Batch& bt, unsigned int* rc32, const float* alpha, const float2* tw,
                                 int* ctl, int* err, int nsm, cudaStream_t st, uint32_t spin_limit = 0);
cudaError_t launch_rc32_to_rc(long n3, const unsigned int* rc32, uint8_t* rc, cudaStream_t st);

// Criterion and adjoint (kernels_adj.cu).
cudaError_t adj_setup(int N);
int adj_zpart_blocks(int N);
cudaError_t launch_cols_a_crit(int N, const Batch& bt, float* C, uint8_t* A, const float* alpha, const float2* tw,
                               cudaStream_t st);
cudaError_t launch_cols_a_adj(int N, const Batch& bt, const float* g, const uint8_t* A, const float* alpha,
                              float* zpart, const float2* tw, cudaStream_t st);
cudaError_t launch_rows_adj_acc(int N, const Batch& bt, float2* acc, const float2* tw, cudaStream_t st);
// The same rules for any box side, as per-element passes over natural-layout
// work boxes after whole-box transforms (the shared-memory transform family).
int adj_elem_blocks();
cudaError_t launch_crit_elem(long n3, const Batch& bt, float* C, uint8_t* A, const float* alpha, cudaStream_t st);
cudaError_t launch_adj_elem(long n3, const Batch& bt, const float* g, const uint8_t* A, const float* alpha,
                            float* zpart, cudaStream_t st);
cudaError_t launch_acc_elem(int N, const Batch& bt, float2* acc, cudaStream_t st);
cudaError_t launch_grad_finish(long n3, const float2* G, const float* alpha, const float* delta, const float* rec0,
                               float r2, float r3, float src_mul, float* gdelta, float* gsrc, cudaStream_t st);
cudaError_t launch_crit_init(long n3, float* C, uint8_t* A, cudaStream_t st);
cudaError_t launch_crit_finalize(long n3, float* C, const uint8_t* A, cudaStream_t st);

// Halo-catalogue source box (kernels_halo.cu): CIC of Rion + block average,
// bit-identical with the reference's serial loop.  halos_dev: nh records
// {float Mass, x, y, z}; fine: N_halo^3 floats; out: N_smooth^3 floats.
// qion != 0: the weight is Rion / qion (sfr, get_SFR.c:119-121); post_div != 0:
// each smoothed cell is then divided by it (get_SFR.c:129-131).
size_t halo_scratch_bytes(long nh);
cudaError_t launch_halo_source(long nh, const void* halos_dev, double z, long N_halo, long N_smooth, float* fine,
                               float* out, void* scratch, size_t scratch_bytes, cudaStream_t st, double qion = 0.0,
                               double post_div = 0.0);
// The same with its scratch in a fixed static device array (no allocation);
// returns an SF21_* status and writes a message into err on failure.
int halo_source_noalloc(double z, long N_halo, long N_smooth, long nh, const void* halos_dev, float* out,
                        cudaStream_t st, char* err, size_t errlen);
// Error text of the context-free entry points (hii_api.cu).
void set_global_error(const char* msg);
// Qion(z) of user_functions.c:84-88 in double, host side (hii_api.cu).
double host_Qion(double z);

// Power spectrum (kernels_pk.cu): window into a complex box, spherical binning
// of |F|^2 over the half-spectrum (per-CTA float sums, exact counts).
int pk_nbins(int N);
int pk_bin_grid(int N);
cudaError_t launch_pk_pack(int N, const float* box, const float* wax, float2* out, cudaStream_t st);
cudaError_t launch_pk_bin(int N, const float2* spec, int nk, float* partials, unsigned long long* counts,
                          cudaStream_t st);

// 21-cm brightness temperature (kernels_t21.cu).
struct T21Args {
  float scale;  // -dg/dt / L^3 / H(z) dx^3 / D(z): Re(unnormalised inverse) -> dv
  float pref;   // 23e-3 (0.7/h) (Omega_b h^2 / 0.02) sqrt(0.15/Omega_m/h^2 (1+z)/10)
  float tcmb;   // Tcmb0 (1 + z)
};
int t21_blocks(long n3);
cudaError_t launch_t21_pack(long n3, const float* delta, float2* out, cudaStream_t st);
// axis: 1 = first index, 2 = second, otherwise the third (Vel_comp)
cudaError_t launch_t21_kfilter(int N, int axis, float2* spec, cudaStream_t st);
// xc, xalpha, tempx: all null (spin temperature >> Tcmb) or all set;
// partials: 2 floats per block (sum of T_b, sum of Tcmb / (1 - t))
cudaError_t launch_t21_finish(long n3, const float2* inv, const float* delta, const float* xhii, const float* xc,
                              const float* xalpha, const float* tempx, const T21Args& ta, float* tb,
                              float* partials, cudaStream_t st);

// Excursion-set halo finder (kernels_hf.cu).
constexpr int HF_KMAX = 4;  // mass pairs per filter-bank pass
struct HfPair {
  float dkRa, dkRb;    // dk R of the two masses (b unused when bits_b is null)
  float thr_a, thr_b;  // candidate <=> filtered value > thr (largest float <= deltaCMZ)
  float2* work;        // N^3 complex work box
  uint32_t* bits_a;    // candidate bit sets, N^3 / 32 words each
  uint32_t* bits_b;
};
struct HfBatch {
  int K;
  float scale;  // dx^3 / L^3 * growth (get_halos.c:225)
  HfPair p[HF_KMAX];
};
// candidate states of the overlap test
constexpr uint8_t HF_UND = 0, HF_PEND_ACC = 1, HF_PEND_REJ = 2, HF_ACC = 3, HF_ACC_FLAGGED = 4, HF_REJ = 5;
cudaError_t hf_setup(int N);
cudaError_t launch_hf_rows_filter(int N, const float2* spec, const HfBatch& hb, const float2* tw, cudaStream_t st);
cudaError_t launch_hf_cols_a_thresh(int N, const HfBatch& hb, const float2* tw, cudaStream_t st);
// column-block-major form: rows_cb -> launch_cols_b_cb (a Batch over the same
// work boxes) -> cols_a_thresh_cb
cudaError_t launch_hf_rows_filter_cb(int N, const float2* spec, const HfBatch& hb, const float2* tw,
                                     cudaStream_t st);
cudaError_t launch_hf_cols_a_thresh_cb(int N, const HfBatch& hb, const float2* tw, cudaStream_t st);
long hf_compact_chunks(long nwords);
cudaError_t launch_bits_count(const uint32_t* W, long nwords, uint32_t* cnt, cudaStream_t st);
cudaError_t launch_scan_counts(uint32_t* cnt, long n, uint32_t* tot, cudaStream_t st);
cudaError_t launch_bits_emit(const uint32_t* W, long nwords, const uint32_t* off, uint32_t* out, cudaStream_t st);
// runs: {di, dj, m, 0}: the cells (i+di, j+dj, p-m .. p+m) of a sphere (or of D)
cudaError_t launch_hf_prefilter(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* runs, int nruns,
                                const uint32_t* FL, uint32_t* UND, uint8_t* status, uint32_t* n_und, cudaStream_t st);
cudaError_t launch_hf_round(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* druns, int ndruns,
                            uint32_t* UND, uint32_t* ACC, uint8_t* status, uint32_t* n_und, cudaStream_t st);
cudaError_t launch_hf_flag_accepted(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* runs,
                                    int nruns, uint32_t* FL, uint8_t* status, cudaStream_t st);
cudaError_t launch_hf_finisher(const uint32_t* list, const uint32_t* n_ptr, int N, const int4* runs, int nruns,
                               uint32_t* FL, uint32_t* ACC, uint8_t* status, cudaStream_t st);
cudaError_t launch_hf_clear(const uint32_t* list, const uint32_t* n_ptr, uint32_t* UND, uint32_t* ACC,
                            cudaStream_t st);
cudaError_t launch_hf_cell(long nwords, const float* delta, float tcell, uint32_t* FL, uint32_t* bits,
                           cudaStream_t st);
cudaError_t launch_hf_records(const uint32_t* idx, long n, int N, float mass, float4* out, cudaStream_t st);

// Subgrid Poisson cycle of the halo finder (kernels_sg.cu).
constexpr int SG_B = 1024;               // stream positions per block
constexpr int SG_THREADS = SG_B / 4;     // 4 consecutive positions per thread
constexpr int SG_LMAX = 64;              // uniforms one draw may consume at most
constexpr int SG_G = 64;                 // children per parent in the entry composition
constexpr int SG_POW2 = 40;              // jump matrices T^(2^k), k < SG_POW2
constexpr int SG_LOCAL = (SG_B + SG_LMAX) / 4;  // jump matrices T^(4 i), i < SG_LOCAL
struct SgArgs {
  uint32_t s0[3];  // taus state before position 0
  uint32_t x1;     // one uniform suffices <=> its 32-bit draw <= x1 (= floor(exp(-mu) 2^32))
  uint64_t emu;    // exp(-mu), double bits
};
// start: 3 words per block (the state at its first position); L: draw length
// per position; LB: SG_B/32 words per block, bit = draw length >= 2
cudaError_t launch_sg_len(long nblocks, const SgArgs& a, const uint32_t* pow2, const uint32_t* local, uint32_t* start,
                          uint8_t* L, uint32_t* LB, uint8_t* X, uint16_t* D, int* err, cudaStream_t st);
// composition scratch: groups (sg_groups(nblocks)) and supergroups
// (sg_groups(groups)) tables (x SG_LMAX), their entries and draw bases
// (sbase: supergroups + 1, the last = draws available), the blocks' entries
struct SgEntryBufs {
  uint8_t *gx, *sx, *gentry, *sentry, *bentry;
  uint32_t *gd, *sd;
  uint64_t *gbase, *sbase, *bbase;
};
long sg_groups(long n);
cudaError_t launch_sg_entries(const uint8_t* X, const uint16_t* D, long nblocks, const SgEntryBufs& eb,
                              cudaStream_t st);
// err: int[3], [0] a draw longer than SG_LMAX, [1] site of an access outside
// its buffer (skipped), [2] its index
cudaError_t launch_sg_walk(int mode, const uint8_t* L, const uint32_t* LB, long nblocks, const uint8_t* bentry,
                           const uint64_t* bbase, uint64_t U, uint32_t* cnt, uint64_t* consumed, uint64_t* dn,
                           uint8_t* dk, uint64_t cap, int* err, cudaStream_t st);
cudaError_t launch_sg_free_count(const uint32_t* FL, long nwords, uint32_t* c, cudaStream_t st);
cudaError_t launch_sg_nn(const uint64_t* dn, const uint8_t* dk, long nd, const uint32_t* FL, const uint32_t* wpre,
                         long nwords, const float* delta, uint64_t growth, uint64_t hbias, uint32_t* cell,
                         uint32_t* nn, int* err, cudaStream_t st);
cudaError_t launch_sg_records(const uint32_t* cell, const uint32_t* nn, const uint32_t* off, long nd, int N,
                              float mass, float4* out, uint64_t cap, int* err, cudaStream_t st);
// exclusive prefix sums of n uint32 (out may equal a); chunk: scan_chunks(n)
// words of scratch; *total (device) receives the sum
long scan_chunks(long n);
cudaError_t launch_scan_u32(const uint32_t* a, long n, uint32_t* out, uint32_t* chunk, uint32_t* total,
                            cudaStream_t st);

// Transforms of any side N = 2^a 3^b 5^c (8 | N, 24 <= N <= 1280) in shared
// memory (kernels_gen.cu), over natural-layout boxes; twiddles: the plain
// table tw[t] = exp(-2 pi i t / N) (gen_twiddles).
struct GenPlan {
  int N;
  int nst;        // stages
  int radix[16];  // radix of each stage (8, 4, 2, 3 or 5)
};
// Register-resident passes for N = 600 (kernels_gen600.cu): 600 = 24 x 25,
// one shared-memory exchange per line; twiddles: the plain table of the
// shared-memory family.  cb: the radius batch's work boxes in the
// column-block-major layout ((c / 8) N + a) N + b) 8 + c mod 8 (rows mode 2
// writes it, the b-axis inverse and the a-axis test pass read it); otherwise
// natural boxes.  launch_gen600_cols_a_test reads the batch in that layout.
bool gen600_supported(int N);
cudaError_t gen600_setup();
cudaError_t launch_gen600_cols(float2* box0, const Batch& bt, int axis, bool inverse, bool cb, const float2* tw,
                               cudaStream_t st);
// rows: mode 0 forward (in -> out, imaginary part times |*alpha|), 1 inverse
// in place (in == out), 2 inverse of the spectrum times the batch's filters
// (in = spectrum -> bt.r[k].work)
cudaError_t launch_gen600_rows(int mode, const float2* in, float2* out, const Batch& bt, const float* alpha,
                               const float2* tw, bool cb, cudaStream_t st);
cudaError_t launch_gen600_cols_a_test(const Batch& bt, uint8_t* rc, const float* alpha, const float2* tw,
                                      cudaStream_t st);
bool gen_supported(int N);
GenPlan gen_plan(int N);
cudaError_t gen_setup(int N);
cudaError_t launch_gen_fwd_rows(const GenPlan& p, const float2* in, float2* out, const float* alpha, const float2* tw,
                                cudaStream_t st);
cudaError_t launch_gen_inv_rows_plain(const GenPlan& p, float2* box, const float2* tw, cudaStream_t st);
cudaError_t launch_gen_inv_rows_filter(const GenPlan& p, const float2* spec, const Batch& bt, const float2* tw,
                                       cudaStream_t st);
cudaError_t launch_gen_hf_rows_filter(const GenPlan& p, const float2* spec, const HfBatch& hb, const float2* tw,
                                      cudaStream_t st);
// strided axis (1 = b, 0 = a) in place: `box`, or the batch's K boxes when box is null
cudaError_t launch_gen_cols(const GenPlan& p, float2* box, const Batch& bt, int axis, bool inverse, const float2* tw,
                            cudaStream_t st);
cudaError_t launch_gen_cols_a_test(const GenPlan& p, const Batch& bt, uint8_t* rc, const float* alpha,
                                   const float2* tw, cudaStream_t st);
// the pair boxes of hb: inverse pass along axis, and with thresholds (a axis) the bit sets
cudaError_t launch_gen_hf_cols(const GenPlan& p, const HfBatch& hb, int axis, bool thresholds, const float2* tw,
                               cudaStream_t st);

// Plain form (kernels_plain.cu).
cudaError_t launch_plain_centres(long n3, const float2* box, const float* alpha, float zmul, float* mask, int* flag,
                                 cudaStream_t st);
cudaError_t launch_plain_pack_sphere(int N, int nmax, const float* mask, const int* flag, float2* out,
                                     cudaStream_t st);
cudaError_t launch_plain_product(int N, const float2* Z, const int* flag, float2* P, cudaStream_t st);
cudaError_t launch_plain_threshold(long n3, const float2* conv, const int* flag, float* bubblef, cudaStream_t st);
cudaError_t launch_plain_paint(int N, int nc, int nmax, const float* mask, float* bubblef, cudaStream_t st);
cudaError_t launch_plain_cap(long n3, const float* fres, float* bubblef, cudaStream_t st);

}  // namespace sf21
