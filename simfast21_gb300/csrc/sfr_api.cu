// C-ABI of the star-formation-rate stage (get_SFR.c:104-148): a context that
// owns the catalogue, the fine grid and the sort scratch, grown on demand, and
// the per-redshift call that fills the SFRD box through the halo-source
// kernels (kernels_halo.cu) with the sfr weight and the dx_halo^3 division.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>

#include "../../include/sf21_sfr.h"
#include "sf21_kernels.h"

using namespace sf21;

namespace {
std::string g_sfr_err;
}  // namespace

struct sf21_sfr_ctx {
  sf21_sfr_config cfg;
  long n3_halo = 0, n3 = 0;
  double dx_halo = 0;
  cudaStream_t stream = nullptr;
  float *d_fine = nullptr, *d_out = nullptr;
  void *d_halos = nullptr, *d_scratch = nullptr;
  size_t scratch_bytes = 0;
  long halo_cap = 0;
  std::string err;
};

#define SCTX_FAIL(ctx, code, ...)          \
  do {                                     \
    char _b[512];                          \
    snprintf(_b, sizeof(_b), __VA_ARGS__); \
    (ctx)->err = _b;                       \
    return (code);                         \
  } while (0)

#define SCTX_CUDA(ctx, call)                                                                                  \
  do {                                                                                                        \
    cudaError_t _e = (call);                                                                                  \
    if (_e != cudaSuccess)                                                                                    \
      SCTX_FAIL(ctx, _e == cudaErrorMemoryAllocation ? SF21_E_ALLOC : SF21_E_CUDA, "%s failed: %s (%s:%d)", \
                #call, cudaGetErrorString(_e), __FILE__, __LINE__);                                           \
  } while (0)

static void free_sctx(sf21_sfr_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->cfg.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* ptrs[] = {c->d_fine, c->d_out, c->d_halos, c->d_scratch};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int sf21_sfr_create(const sf21_sfr_config* cfg, sf21_sfr_ctx** out) {
  g_sfr_err.clear();
  if (!cfg || !out) {
    g_sfr_err = "NULL config or output pointer";
    return SF21_E_ARG;
  }
  *out = nullptr;
  // smooth_box refuses N_smoothed > N_halo (auxiliary.c:651-654); the cell
  // keys of the deposit are 64-bit, the grids at most 2048^3
  if (cfg->N_halo < 1 || cfg->N_smoothed < 1 || cfg->N_halo > 2048 || cfg->N_smoothed > cfg->N_halo) {
    g_sfr_err = "need 1 <= N_smoothed <= N_halo <= 2048";
    return SF21_E_ARG;
  }
  if (!(cfg->L > 0)) {
    g_sfr_err = "L must be positive";
    return SF21_E_ARG;
  }
  sf21_sfr_ctx* c = new sf21_sfr_ctx();
  c->cfg = *cfg;
  c->n3_halo = cfg->N_halo * cfg->N_halo * cfg->N_halo;
  c->n3 = cfg->N_smoothed * cfg->N_smoothed * cfg->N_smoothed;
  c->dx_halo = cfg->L / cfg->N_halo;  // global_dx_halo, Input_variables.c:128
#define SCREATE(call)                                                                     \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) {                                                              \
      g_sfr_err = std::string(#call) + " failed: " + cudaGetErrorString(_e);             \
      free_sctx(c);                                                                       \
      return _e == cudaErrorMemoryAllocation ? SF21_E_ALLOC : SF21_E_CUDA;                \
    }                                                                                     \
  } while (0)
  SCREATE(cudaSetDevice(cfg->device));
  SCREATE(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  SCREATE(dev_malloc(&c->d_fine, sizeof(float) * c->n3_halo));
  SCREATE(dev_malloc(&c->d_out, sizeof(float) * c->n3));
#undef SCREATE
  *out = c;
  return SF21_OK;
}

extern "C" void sf21_sfr_destroy(sf21_sfr_ctx* c) { free_sctx(c); }

extern "C" const char* sf21_sfr_last_error(const sf21_sfr_ctx* c) { return c ? c->err.c_str() : g_sfr_err.c_str(); }

// Grows the catalogue and scratch buffers to hold nhalos records.
static int ensure_halo_cap(sf21_sfr_ctx* c, long nhalos) {
  if (nhalos <= c->halo_cap) return SF21_OK;
  if (c->d_halos) cudaFree(c->d_halos);
  if (c->d_scratch) cudaFree(c->d_scratch);
  c->d_halos = nullptr;
  c->d_scratch = nullptr;
  c->halo_cap = 0;
  long cap = nhalos + nhalos / 4 + 1024;
  if (cap >= (1L << 28)) cap = (1L << 28) - 1;
  SCTX_CUDA(c, dev_malloc(&c->d_halos, (size_t)cap * 16));
  c->scratch_bytes = halo_scratch_bytes(cap);
  SCTX_CUDA(c, dev_malloc(&c->d_scratch, c->scratch_bytes));
  c->halo_cap = cap;
  return SF21_OK;
}

static int enqueue_sfr(sf21_sfr_ctx* c, double z, long nhalos, const void* halos_dev, float* out_dev,
                       cudaStream_t st) {
  // sfr(M, z) = Rion(M, z) / Qion(z) (user_functions.c:71-75) into CIC's
  // float weight; sfrd = smoothed / pow(dx_halo, 3) (get_SFR.c:129-131)
  const double qion = host_Qion(z);
  const double dx3 = pow(c->dx_halo, 3);
  SCTX_CUDA(c, launch_halo_source(nhalos, halos_dev, z, c->cfg.N_halo, c->cfg.N_smoothed, c->d_fine, out_dev,
                                  c->d_scratch, c->scratch_bytes, st, qion, dx3));
  return SF21_OK;
}

static int check_catalogue(sf21_sfr_ctx* c, long nhalos, const void* halos) {
  if (nhalos < 0 || (nhalos > 0 && !halos)) SCTX_FAIL(c, SF21_E_ARG, "bad halo catalogue");
  if (nhalos >= (1L << 28)) SCTX_FAIL(c, SF21_E_UNSUPPORTED, "2^28 halos or more (8 CIC entries each, int count)");
  return SF21_OK;
}

extern "C" int sf21_sfr_box(sf21_sfr_ctx* c, double z, long nhalos, const void* halos, float* sfrd,
                            double* sfrd_mean) {
  if (!c) return SF21_E_ARG;
  if (!sfrd) SCTX_FAIL(c, SF21_E_ARG, "NULL output box");
  int rc;
  if ((rc = check_catalogue(c, nhalos, halos))) return rc;
  SCTX_CUDA(c, cudaSetDevice(c->cfg.device));
  if ((rc = ensure_halo_cap(c, nhalos))) return rc;
  if (nhalos > 0)
    SCTX_CUDA(c, cudaMemcpyAsync(c->d_halos, halos, (size_t)nhalos * 16, cudaMemcpyHostToDevice, c->stream));
  if ((rc = enqueue_sfr(c, z, nhalos, c->d_halos, c->d_out, c->stream))) return rc;
  SCTX_CUDA(c, cudaMemcpyAsync(sfrd, c->d_out, sizeof(float) * c->n3, cudaMemcpyDeviceToHost, c->stream));
  SCTX_CUDA(c, cudaStreamSynchronize(c->stream));
  if (sfrd_mean) {
    // get_SFR.c:141-145: serial double sum in index order
    double s = 0.0;
    for (long i = 0; i < c->n3; ++i) s += sfrd[i];
    *sfrd_mean = s / c->n3;
  }
  return SF21_OK;
}

extern "C" int sf21_sfr_box_device(sf21_sfr_ctx* c, double z, long nhalos, const void* halos_dev, float* sfrd_dev,
                                   void* stream) {
  if (!c) return SF21_E_ARG;
  if (!sfrd_dev) SCTX_FAIL(c, SF21_E_ARG, "NULL output box");
  int rc;
  if ((rc = check_catalogue(c, nhalos, halos_dev))) return rc;
  SCTX_CUDA(c, cudaSetDevice(c->cfg.device));
  if ((rc = ensure_halo_cap(c, nhalos))) return rc;
  return enqueue_sfr(c, z, nhalos, halos_dev, sfrd_dev, (cudaStream_t)stream);
}
