// C-ABI of the HII filter bank (include/sf21_hii.h): context, device
// buffers, per-redshift scalars and the launch schedule.
//
// Schedule of one redshift (get_HIIbubbles.c:215-471), all on one stream:
//   prologue            rec0, fresid, packed (rec0, ion)   (:216-225, :272-274)
//   alpha               norm balance of the packed transform
//   forward 3D FFT      spectrum of the packed box          (:290-291)
//   for each set:
//     rc := none
//     for each batch of up to K radii (descending R):     (:298-461)
//       c-axis inverse with the top-hat filter of K radii -> K work boxes
//       b-axis inverse of the K boxes
//       a-axis inverse + centre test + first-hit update of rc
//     dilation of the first-hit field + single-cell fill + cap -> xHII (:281-288, :358-393, :427-458, :466-471)
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <stdlib.h>

#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sf21_hii.h"
#include "sf21_kernels.h"

using namespace sf21;

namespace {

const double kPI = 3.1415926535897932385E0;  // Input_variables.h:10
const double kCM_PER_MPC = 3.0857e24;         // user_functions.c:26

uint64_t dbits(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
}

// ---- per-redshift scalars, evaluated on the host with the C library's pow
// and in the reference's operation order (user_functions.c:59-97) ---------
double host_G_H(double z) {
  double lo = -4.37152818e-05 * pow(z, 5.) + 1.64394635e-03 * pow(z, 4.) -
              2.03044756e-02 * pow(z, 3.);
  double hi = 7.18335221e-02 * pow(z, 2.) - 8.85791388e-02 * z - 1.20887500e+01;
  return 4.19232273531e-13 / pow(10.0, lo + hi);
}

struct SetInfo {
  double fesc, Rmax;
  int Nbins;
  std::vector<double> R;     // radii, loop order
  int n_fft;                 // radii with R >= 2 dx
  std::vector<int> nmax;     // largest n with sqrt(n)*dx <= R
  int vmax;
  int* d_nmax = nullptr;
};

}  // namespace

namespace sf21 {
// Allocation-failure injection (sf21_hii_inject_alloc_failure): the n-th
// device allocation after arming fails once.
static std::atomic<long> g_fail_alloc_in{0};

cudaError_t dev_malloc(void** p, size_t bytes) {
  long n = g_fail_alloc_in.load();
  while (n > 0 && !g_fail_alloc_in.compare_exchange_weak(n, n - 1)) {
  }
  if (n == 1) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

// Qion(z) (user_functions.c:84-88), shared with the star-formation-rate stage.
double host_Qion(double z) { return pow(10.0, 2.05707274e-02 * z + 5.29944413e+01) / 1.e+45; }
}  // namespace sf21

// Radius pipelines: 1 three axis passes, 2 plane clusters + kx pass,
// 3 TMA ky + kx pass, 4 TMA ky + TMA kx, and over column-block-major work
// boxes: 5 three axis passes, 6 TMA ky + kx pass, 7 TMA ky + TMA kx,
// 8 c-axis pass + one persistent ky/kx launch handing each slab over in L2.
constexpr int NPATH = 8;

struct sf21_hii_ctx {
  int device = 0;
  bool gen = false;  // side not a power of two: shared-memory transforms (kernels_gen.cu), pipeline 1 only
  GenPlan gp = {};
  long N = 0, N_halo = 0, n3 = 0;
  double L = 0, hubble = 0, dx = 0, dk = 0;
  int K = 8;
  int path = 1;             // 1 = three axis passes, 2 = plane clusters + kx pass,
                            // 3 = three axis passes, ky pass TMA-pipelined,
                            // 4 = three axis passes, ky and kx passes TMA-pipelined
  double tune_ms[NPATH + 1] = {};
  float2* d_work_base = nullptr;  // K consecutive work boxes
  // CUDA graph of the per-redshift schedule of run_z_device (replayed while
  // z, the source kind, the buffers and the stream stay the same)
  bool use_graph = true;
  cudaGraphExec_t gexec = nullptr;
  struct GraphKey {
    double z;
    int kind;
    const void *delta, *src, *xhii;
    cudaStream_t st;
  } gkey = {0, -1, nullptr, nullptr, nullptr, nullptr};
  PipeMaps pmaps;
  int* d_err = nullptr;
  int* d_ctl = nullptr;     // work-queue control block of pipeline 8
  unsigned int* d_rc32 = nullptr;  // pipeline 8: 32-bit first-hit box (atomicMin), folded into d_rc per set
  uint32_t wait_limit = 0;  // polls per bounded device wait (0 = the kernels' default)
  int nsm = 0;
  std::vector<SetInfo> sets;
  cudaStream_t stream = nullptr;
  // host-buffer entry points: downloads of set s overlap the compute of set
  // s + 1 (second stream, two staging boxes used in turn)
  cudaStream_t copy_stream = nullptr;
  float* d_xhii2 = nullptr;
  cudaEvent_t ev_done[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
  float *d_delta = nullptr, *d_src = nullptr, *d_rec0 = nullptr, *d_fres = nullptr;
  uint64_t* d_chain = nullptr;  // source chain before zeta (double bits), per redshift
  float2* d_om = nullptr;       // 1 - fresid rounded down / to nearest, per redshift
  float *d_partials = nullptr, *d_alpha = nullptr, *d_xhii = nullptr;
  // criterion / adjoint buffers (allocated on first use)
  float* d_C = nullptr;
  uint8_t* d_A = nullptr;
  float2* d_acc = nullptr;
  float* d_zpart = nullptr;
  float *d_g = nullptr, *d_gd = nullptr, *d_gs = nullptr;
  int crit_set = -1;
  double crit_z = 0;
  // halo-catalogue source buffers (allocated / grown on use)
  void* d_halos = nullptr;
  long halo_cap = 0;
  float* d_fine = nullptr;
  // power-spectrum buffers (allocated on first use)
  float2* d_pk = nullptr;
  float* d_pk_w = nullptr;
  float* d_pk_part = nullptr;
  unsigned long long* d_pk_cnt = nullptr;
  // 21-cm brightness-temperature buffers (allocated on first use)
  float* d_t21 = nullptr;  // xc, xalpha, TK, T_b boxes
  float* d_t21_part = nullptr;
  void* d_hscratch = nullptr;
  size_t hscratch_bytes = 0;
  // plain-form buffers (allocated on first use)
  float* d_mask = nullptr;
  int* d_flag = nullptr;
  float2* d_box2 = nullptr;
  float2 *d_spec = nullptr, *d_tw = nullptr;
  std::vector<float2*> d_work;
  uint8_t* d_rc = nullptr;
  PrologueArgs pa;   // scalars of the redshift being processed (kernel arguments)
  int pro_blocks = 0;
  std::string err;
  // optional per-kernel timing (CUDA events on the launch stream)
  bool prof = false;
  std::vector<cudaEvent_t> ev;
  size_t ev_used = 0;
  struct Span { int kind, a, b; };
  std::vector<Span> spans;
  double prof_ms[32] = {0};
  long prof_n[32] = {0};
};

// Kernel kinds reported by sf21_hii_profile_read, in this order.
static const char* kKindNames[] = {"prologue", "alpha", "fwd_rows", "fwd_cols_b", "fwd_cols_a",
                                   "inv_rows_filter", "inv_cols_b", "inv_cols_a_test", "dt_a",
                                   "dt_b", "dt_c_finish", "inv_plane_filter", "crit_cols_a",
                                   "adj_cols_a", "adj_cols_b_fwd", "adj_rows_acc", "adj_final",
                                   "finish_prep", "inv_cols_ba_fused"};
enum { KD_PRO, KD_ALPHA, KD_FROWS, KD_FCB, KD_FCA, KD_IROWS, KD_ICB, KD_ICA, KD_DTR, KD_DTB, KD_DTA, KD_PLANE,
       KD_CRIT, KD_ADJA, KD_ADJB, KD_ADJR, KD_ADJF, KD_PREP, KD_FUSED, KD_COUNT };

// Records an event on st when timing is on; returns its index (or -1).
static int mark(sf21_hii_ctx* c, cudaStream_t st) {
  if (!c->prof) return -1;
  if (c->ev_used == c->ev.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    c->ev.push_back(e);
  }
  cudaEventRecord(c->ev[c->ev_used], st);
  return (int)c->ev_used++;
}
static void span(sf21_hii_ctx* c, int kind, int a, int b) {
  if (c->prof && a >= 0 && b >= 0) c->spans.push_back({kind, a, b});
}

static std::string g_create_err;

// ---- autotuner cache --------------------------------------------------------
// One JSON object per line, {"key": "<device>|N=<N>|K=<K>", "ms": [t1, ..., t7]}
// (milliseconds of one batch per radius pipeline, 0 = not available), in
// $SF21_TUNE_CACHE, else $XDG_CACHE_HOME/simfast21_gb300/tune.jsonl, else
// ~/.cache/simfast21_gb300/tune.jsonl.  SF21_RETUNE=1 ignores the cache (and
// rewrites the entry).  A missing or unreadable cache only means tuning again.
static std::string tune_cache_path() {
  if (const char* p = getenv("SF21_TUNE_CACHE")) return p;
  std::string dir;
  if (const char* x = getenv("XDG_CACHE_HOME")) dir = x;
  else if (const char* h = getenv("HOME")) dir = std::string(h) + "/.cache";
  else return "";
  return dir + "/simfast21_gb300/tune.jsonl";
}

static std::string tune_key(int device, long N, int K) {
  cudaDeviceProp pr;
  char b[512];
  if (cudaGetDeviceProperties(&pr, device) != cudaSuccess) return "";
  snprintf(b, sizeof b, "%s sm_%d%d x%d|N=%ld|K=%d", pr.name, pr.major, pr.minor, pr.multiProcessorCount, N, K);
  for (char* q = b; *q; ++q)
    if (*q == '"' || *q == '\\') *q = '_';
  return b;
}

static bool tune_cache_lookup(const std::string& key, double* ms, int npath) {
  const char* re = getenv("SF21_RETUNE");
  if (key.empty() || (re && re[0] == '1')) return false;
  const std::string path = tune_cache_path();
  FILE* f = path.empty() ? nullptr : fopen(path.c_str(), "r");
  if (!f) return false;
  char line[2048];
  bool found = false;
  const std::string want = "{\"key\": \"" + key + "\", \"ms\": [";
  while (fgets(line, sizeof line, f)) {
    if (strncmp(line, want.c_str(), want.size()) != 0) continue;
    double v[16];
    const char* q = line + want.size();
    int n = 0;
    while (n < npath) {
      char* end = nullptr;
      v[n] = strtod(q, &end);
      if (end == q) break;
      ++n;
      q = end;
      while (*q == ',' || *q == ' ') ++q;
    }
    if (n != npath) continue;
    bool any = false;
    for (int p = 1; p <= npath; ++p) {
      ms[p] = v[p - 1] > 0 ? v[p - 1] : 1e30;
      any |= v[p - 1] > 0;
    }
    found = any;  // the last matching line wins
  }
  fclose(f);
  return found;
}

static void tune_cache_store(const std::string& key, const double* ms, int npath) {
  const std::string path = tune_cache_path();
  if (key.empty() || path.empty()) return;
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {  // create the directory (and its parent) if needed
    const std::string dir = path.substr(0, slash);
    const size_t up = dir.rfind('/');
    if (up != std::string::npos) mkdir(dir.substr(0, up).c_str(), 0755);
    mkdir(dir.c_str(), 0755);
  }
  FILE* f = fopen(path.c_str(), "a");
  if (!f) return;
  fprintf(f, "{\"key\": \"%s\", \"ms\": [", key.c_str());
  for (int p = 1; p <= npath; ++p) fprintf(f, "%s%.6g", p > 1 ? ", " : "", ms[p] < 1e29 ? ms[p] : 0.0);
  fprintf(f, "]}\n");
  fclose(f);
}

#define CTX_FAIL(ctx, code, ...)                                  \
  do {                                                            \
    char _b[512];                                                 \
    snprintf(_b, sizeof(_b), __VA_ARGS__);                        \
    (ctx)->err = _b;                                              \
    return (code);                                                \
  } while (0)

#define CTX_CUDA(ctx, call)                                                                        \
  do {                                                                                             \
    cudaError_t _e = (call);                                                                       \
    if (_e != cudaSuccess)                                                                         \
      CTX_FAIL(ctx, _e == cudaErrorMemoryAllocation ? SF21_E_ALLOC : SF21_E_CUDA, "%s failed: %s (%s:%d)", \
               #call, cudaGetErrorString(_e), __FILE__, __LINE__);                                 \
  } while (0)

static int nmax_of(double R, double dx) {
  long n = (long)floor((R / dx) * (R / dx));
  if (n < 0) n = 0;
  while (n > 0 && !(sqrt((double)n) * dx <= R)) --n;
  while (sqrt((double)(n + 1)) * dx <= R) ++n;
  return (int)n;
}

static void build_set(SetInfo& s, double dx) {
  // bfactor (:192) and the two loops (:299, :397, :402, :461)
  const double b = pow(10.0, log10(s.Rmax / dx) / s.Nbins);
  double R = s.Rmax;
  s.R.clear();
  while (R >= 2 * dx) {
    s.R.push_back(R);
    R /= b;
  }
  s.n_fft = (int)s.R.size();
  while (R >= dx) {
    s.R.push_back(R);
    R /= b;
  }
  s.nmax.resize(s.R.size());
  s.vmax = 0;
  for (size_t i = 0; i < s.R.size(); ++i) {
    s.nmax[i] = nmax_of(s.R[i], dx);
    if (s.nmax[i] > s.vmax) s.vmax = s.nmax[i];
  }
}

static void free_ctx(sf21_hii_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  void* ptrs[] = {c->d_delta, c->d_src, c->d_rec0, c->d_fres, c->d_partials, c->d_alpha,
                  c->d_xhii, c->d_spec, c->d_tw, c->d_rc, c->d_mask, c->d_flag, c->d_box2,
                  c->d_C, c->d_A, c->d_acc, c->d_zpart, c->d_g, c->d_gd, c->d_gs, c->d_halos, c->d_fine,
                  c->d_hscratch, c->d_chain, c->d_om, c->d_xhii2, c->d_pk, c->d_pk_w, c->d_pk_part,
                  c->d_pk_cnt, c->d_t21, c->d_t21_part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->d_work_base) cudaFree(c->d_work_base);
  if (c->d_err) cudaFree(c->d_err);
  if (c->d_ctl) cudaFree(c->d_ctl);
  if (c->d_rc32) cudaFree(c->d_rc32);
  for (SetInfo& s : c->sets)
    if (s.d_nmax) cudaFree(s.d_nmax);
  for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  for (int i = 0; i < 2; ++i) {
    if (c->ev_done[i]) cudaEventDestroy(c->ev_done[i]);
    if (c->ev_copied[i]) cudaEventDestroy(c->ev_copied[i]);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

static int prologue_args(sf21_hii_ctx* c, double z, int kind, PrologueArgs* pa) {
  memset(pa, 0, sizeof(*pa));
  pa->one_plus_z_cubed = dbits(pow(1. + z, 3.0));
  pa->g_h = dbits(host_G_H(z));
  pa->rec1 = dbits(1.e-24 * 9.84815696 * pow((1.0 + z), 5.06773134));
  pa->dvv = dbits(pow(c->L * kCM_PER_MPC / c->N / c->hubble / (1. + z), 3.0));
  pa->c_resid = dbits(1.881e-7);
  pa->r2 = dbits(1.76105133);
  pa->r3 = dbits(0.81722878);
  pa->v_norm = dbits(1.e+45);
  pa->r2c = sd_divc_prepare(pa->r2);
  pa->v_normc = sd_divc_prepare(pa->v_norm);
  if (kind == SF21_SRC_SFRD) {
    // halo_map*dx*dx*dx*Qion(z) [*fesc]  (:273)
    pa->src_mul[0] = pa->src_mul[1] = pa->src_mul[2] = dbits(c->dx);
    pa->src_mul[3] = dbits(host_Qion(z));
    pa->n_src_mul = 4;
  } else if (kind == SF21_SRC_RION) {
    // halo_map*pow(dx_s/dx_h,3) [*fesc]  (:258)
    const double dxh = c->L / c->N_halo;
    pa->src_mul[0] = dbits(pow(c->dx / dxh, 3));
    pa->n_src_mul = 1;
  } else {
    CTX_FAIL(c, SF21_E_ARG, "unknown src_kind %d", kind);
  }
  pa->rf = rrec_fast_prepare(pa->rec1, pa->dvv, pa->v_norm, pa->r2, pa->r3);
  const sd_t resid[3] = {pa->c_resid, pa->one_plus_z_cubed, pa->g_h};
  pa->pf_resid = prod_fast_prepare(resid, 3);
  pa->pf_src = prod_fast_prepare(pa->src_mul, pa->n_src_mul);
  return SF21_OK;
}

static int enqueue_batch(sf21_hii_ctx* c, const Batch& bt, cudaStream_t st);
static int check_device_flag(sf21_hii_ctx* c);

extern "C" int sf21_hii_create(const sf21_hii_config* cfg, sf21_hii_ctx** out) {
  if (!out) return SF21_E_ARG;
  *out = nullptr;
  g_create_err.clear();
  if (!cfg || cfg->nsets < 1 || !cfg->sets) {
    g_create_err = "config must have nsets >= 1 and a sets array";
    return SF21_E_ARG;
  }
  const long N = cfg->N;
  const bool pow2 = N >= 16 && N <= 1024 && !(N & (N - 1));
  if (!pow2 && !gen_supported((int)N)) {
    g_create_err = "N_smoothed must be a power of two between 16 and 1024, or a product of 2, 3 and 5 that 8 divides, "
                   "from 24 to 1280";
    return SF21_E_UNSUPPORTED;
  }
  if (!(cfg->L > 0) || !(cfg->hubble > 0)) {
    g_create_err = "L and hubble must be positive";
    return SF21_E_ARG;
  }
  sf21_hii_ctx* c = new sf21_hii_ctx();
  c->device = cfg->device;
  c->N = N;
  c->N_halo = cfg->N_halo > 0 ? cfg->N_halo : N;
  c->n3 = N * N * N;
  c->L = cfg->L;
  c->hubble = cfg->hubble;
  c->dx = cfg->L / N;                 // Input_variables.c:129
  c->dk = 2 * kPI / cfg->L;           // Input_variables.c:127
  for (int s = 0; s < cfg->nsets; ++s) {
    SetInfo si;
    si.fesc = cfg->sets[s].fesc;
    si.Rmax = cfg->sets[s].Rmax;
    si.Nbins = cfg->sets[s].Nbins;
    if (si.Nbins < 1 || !(si.Rmax > 0) || !(si.fesc >= 0)) {
      g_create_err = "set " + std::to_string(s) + ": need Nbins >= 1, Rmax > 0, fesc >= 0";
      delete c;
      return SF21_E_ARG;
    }
    build_set(si, c->dx);
    if (si.R.size() > 254) {
      g_create_err = "set " + std::to_string(s) + ": more than 254 radii";
      delete c;
      return SF21_E_UNSUPPORTED;
    }
    c->sets.push_back(si);
  }
  const size_t box_c = sizeof(float2) * c->n3, box_f = sizeof(float) * c->n3;
  int K = cfg->kmax > 0 ? cfg->kmax : KMAX;
  if (K > KMAX) K = KMAX;
  c->K = K;
  c->use_graph = cfg->graph >= 0;
#define CREATE_CUDA(call)                                                                   \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess) {                                                                \
      g_create_err = std::string(#call) + " failed: " + cudaGetErrorString(_e);             \
      free_ctx(c);                                                                          \
      return _e == cudaErrorMemoryAllocation ? SF21_E_ALLOC : SF21_E_CUDA;                  \
    }                                                                                       \
  } while (0)
  CREATE_CUDA(cudaSetDevice(c->device));
  CREATE_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->gen = !pow2;
  if (c->gen) {
    c->gp = gen_plan((int)N);
    CREATE_CUDA(gen_setup((int)N));
    if (gen600_supported((int)N)) CREATE_CUDA(gen600_setup());
  } else {
    CREATE_CUDA(fft_setup((int)N));
    CREATE_CUDA(cb_setup((int)N));
    CREATE_CUDA(adj_setup((int)N));
  }
  CREATE_CUDA(dt_setup((int)N));
  CREATE_CUDA(dev_malloc(&c->d_delta, box_f));
  CREATE_CUDA(dev_malloc(&c->d_src, box_f));
  CREATE_CUDA(dev_malloc(&c->d_rec0, box_f));
  CREATE_CUDA(dev_malloc(&c->d_fres, box_f));
  CREATE_CUDA(dev_malloc(&c->d_chain, sizeof(uint64_t) * c->n3));
  CREATE_CUDA(dev_malloc(&c->d_om, sizeof(float2) * c->n3));
  CREATE_CUDA(dev_malloc(&c->d_xhii, box_f));
  CREATE_CUDA(dev_malloc(&c->d_spec, box_c));
  CREATE_CUDA(dev_malloc(&c->d_rc, c->n3));
  c->d_work.assign(K, nullptr);
  CREATE_CUDA(dev_malloc(&c->d_work_base, box_c * K));
  for (int k = 0; k < K; ++k) c->d_work[k] = c->d_work_base + (size_t)k * c->n3;
  CREATE_CUDA(dev_malloc(&c->d_err, sizeof(int)));
  CREATE_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
  CREATE_CUDA(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
  c->pro_blocks = prologue_blocks(c->n3);
  CREATE_CUDA(dev_malloc(&c->d_partials, sizeof(float) * 2 * c->pro_blocks));
  CREATE_CUDA(dev_malloc(&c->d_alpha, sizeof(float)));
  // twiddles exp(-2 pi i t / N) in double, rounded once (stage layout for the
  // register transforms, plain table for the shared-memory ones)
  std::vector<float2> tw(N);
  if (c->gen) {
    for (long t = 0; t < N; ++t) {
      const double ang = -2.0 * kPI * t / N;
      tw[t] = make_float2((float)cos(ang), (float)sin(ang));
    }
  } else {
    std::vector<double> tre(N), tim(N);
    twiddle_layout((int)N, tre.data(), tim.data());
    for (long t = 0; t < N; ++t) tw[t] = make_float2((float)tre[t], (float)tim[t]);
  }
  CREATE_CUDA(dev_malloc(&c->d_tw, sizeof(float2) * N));
  CREATE_CUDA(cudaMemcpy(c->d_tw, tw.data(), sizeof(float2) * N, cudaMemcpyHostToDevice));
  for (SetInfo& s : c->sets) {
    CREATE_CUDA(dev_malloc(&s.d_nmax, sizeof(int) * s.nmax.size()));
    CREATE_CUDA(cudaMemcpy(s.d_nmax, s.nmax.data(), sizeof(int) * s.nmax.size(), cudaMemcpyHostToDevice));
  }
  // path: explicit, or tuned by timing one K-radius batch of each variant
  const bool can_plane = !c->gen && plane_supported((int)N) && plane_setup((int)N) == cudaSuccess &&
                         plane_max_active_clusters((int)N) > 0;
  bool can_pipe = false;
  if (!c->gen && pipe_supported((int)N) && pipe_setup((int)N) == cudaSuccess &&
      pipe_make_maps((int)N, &c->pmaps, K, c->d_work_base) == cudaSuccess)
    can_pipe = true;
  bool can_fused = false;
  if (!c->gen && fused_supported((int)N) && fused_setup((int)N) == cudaSuccess &&
      dev_malloc(&c->d_ctl, sizeof(int) * fused_ctl_ints((int)N)) == cudaSuccess &&
      dev_malloc(&c->d_rc32, sizeof(unsigned int) * c->n3) == cudaSuccess)
    can_fused = true;
  cudaGetLastError();
  const int want = cfg->path;
  if ((want == 2 && !can_plane) || ((want == 3 || want == 4 || want == 6 || want == 7) && !can_pipe) ||
      (want == 8 && !can_fused) ||
      (c->gen && want > 1) || want < 0 || want > NPATH) {
    g_create_err = "requested radius pipeline not available for this box on this device";
    free_ctx(c);
    return SF21_E_UNSUPPORTED;
  }
  c->path = want ? want : 1;
  // a tuning result cached for this device, box size and batch size skips the timing
  // Autotuner: the radius pipeline and the radii per spectrum read K.  For
  // each candidate K (the cap, and 6 and 4 below it unless the caller fixed
  // kmax) one K-radius batch of every available pipeline is timed (or the
  // timings are read from the per-device cache); the (pipeline, K) with the
  // least time per radius wins.
  auto available = [&](int p) {
    return !((p == 2 && !can_plane) || ((p == 3 || p == 4 || p == 6 || p == 7) && !can_pipe) ||
             (p == 8 && !can_fused));
  };
  if (want == 0 && (can_plane || can_pipe || can_fused)) {
    std::vector<int> kcands = {K};
    if (cfg->kmax <= 0)
      for (int kc : {6, 4})
        if (kc < K) kcands.push_back(kc);
    double best_per_radius = 1e30;
    int best_path = 1, best_K = K;
    double best_ms[NPATH + 1];
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    bool zeroed = false;
    for (int Kc : kcands) {
      double ms_p[NPATH + 1];
      for (int p = 0; p <= NPATH; ++p) ms_p[p] = 1e30;
      const std::string tkey = tune_key(c->device, N, Kc);
      if (!tune_cache_lookup(tkey, ms_p, NPATH)) {
        if (!zeroed) {
          CREATE_CUDA(cudaMemsetAsync(c->d_spec, 0, box_c, c->stream));
          CREATE_CUDA(cudaMemsetAsync(c->d_alpha, 0, sizeof(float), c->stream));
          CREATE_CUDA(cudaEventCreate(&t0));
          CREATE_CUDA(cudaEventCreate(&t1));
          zeroed = true;
        }
        Batch bt;
        memset(&bt, 0, sizeof(bt));
        bt.K = Kc;
        bt.zmul = 1.0f;
        for (int k = 0; k < Kc; ++k) {
          bt.r[k].dkR = (float)(c->dk * c->dx * (2.0 + k));
          bt.r[k].ridx = k;
          bt.r[k].work = c->d_work[k];
        }
        for (int p = 1; p <= NPATH; ++p) {
          if (!available(p)) continue;
          c->path = p;
          for (int rep = 0; rep < 4; ++rep) {
            CREATE_CUDA(cudaEventRecord(t0, c->stream));
            if (enqueue_batch(c, bt, c->stream) != SF21_OK) {
              g_create_err = c->err;
              cudaEventDestroy(t0);
              cudaEventDestroy(t1);
              free_ctx(c);
              return SF21_E_CUDA;
            }
            CREATE_CUDA(cudaEventRecord(t1, c->stream));
            CREATE_CUDA(cudaEventSynchronize(t1));
            float ms = 0.f;
            CREATE_CUDA(cudaEventElapsedTime(&ms, t0, t1));
            if (rep > 0 && ms < ms_p[p]) ms_p[p] = ms;  // the first run warms up
          }
        }
        int err_flag = 0;
        CREATE_CUDA(cudaMemcpy(&err_flag, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (err_flag) {
          g_create_err = "a bounded device wait expired while tuning";
          if (t0) cudaEventDestroy(t0);
          if (t1) cudaEventDestroy(t1);
          free_ctx(c);
          return SF21_E_TIMEOUT;
        }
        tune_cache_store(tkey, ms_p, NPATH);
      }
      for (int p = 1; p <= NPATH; ++p) {
        if (!available(p) || !(ms_p[p] < 1e29)) continue;
        if (ms_p[p] / Kc < best_per_radius) {
          best_per_radius = ms_p[p] / Kc;
          best_path = p;
          best_K = Kc;
          for (int q = 0; q <= NPATH; ++q) best_ms[q] = ms_p[q];
        }
      }
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    c->path = best_path;
    c->K = best_K;
    if (best_per_radius < 1e29)
      for (int p = 0; p <= NPATH; ++p) c->tune_ms[p] = best_ms[p];
  }
#undef CREATE_CUDA
  *out = c;
  return SF21_OK;
}

extern "C" int sf21_hii_destroy(sf21_hii_ctx* ctx) {
  free_ctx(ctx);
  return SF21_OK;
}

namespace sf21 {
// Error text of the context-free entry points, read with sf21_hii_last_error(NULL).
void set_global_error(const char* msg) { g_create_err = msg; }
}  // namespace sf21

extern "C" const char* sf21_hii_last_error(const sf21_hii_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_create_err.c_str();
}

extern "C" int sf21_hii_radii(const sf21_hii_ctx* ctx, int set, double* R, int cap, int* n_fft) {
  if (!ctx || set < 0 || set >= (int)ctx->sets.size()) return -SF21_E_ARG;
  const SetInfo& s = ctx->sets[set];
  for (int i = 0; i < (int)s.R.size() && i < cap; ++i) R[i] = s.R[i];
  if (n_fft) *n_fft = s.n_fft;
  return (int)s.R.size();
}

// ---- transform passes: register kernels (power-of-two sides) or shared-memory
// kernels (other sides), same arguments ------------------------------------
static cudaError_t x_fwd_rows(sf21_hii_ctx* c, const float2* in, float2* out, const float* alpha, cudaStream_t st) {
  Batch none;
  memset(&none, 0, sizeof(none));
  if (c->gen && gen600_supported((int)c->N)) return launch_gen600_rows(0, in, out, none, alpha, c->d_tw, false, st);
  return c->gen ? launch_gen_fwd_rows(c->gp, in, out, alpha, c->d_tw, st)
                : launch_fwd_rows((int)c->N, in, out, alpha, c->d_tw, st);
}
static cudaError_t x_inv_rows_plain(sf21_hii_ctx* c, float2* box, cudaStream_t st) {
  Batch none;
  memset(&none, 0, sizeof(none));
  if (c->gen && gen600_supported((int)c->N)) return launch_gen600_rows(1, box, box, none, nullptr, c->d_tw, false, st);
  return c->gen ? launch_gen_inv_rows_plain(c->gp, box, c->d_tw, st) : launch_inv_rows_plain((int)c->N, box, c->d_tw, st);
}
// cb: the radius pipeline's batch in the column-block-major layout (N = 600 only)
static cudaError_t x_inv_rows_filter(sf21_hii_ctx* c, const float2* spec, const Batch& bt, cudaStream_t st,
                                     bool cb = false) {
  if (c->gen && gen600_supported((int)c->N)) return launch_gen600_rows(2, spec, nullptr, bt, nullptr, c->d_tw, cb, st);
  return c->gen ? launch_gen_inv_rows_filter(c->gp, spec, bt, c->d_tw, st)
                : launch_inv_rows_filter((int)c->N, spec, bt, c->d_tw, st);
}
// box, or (box null) the batch's nbox = bt.K boxes
static cudaError_t x_cols(sf21_hii_ctx* c, float2* box, const Batch& bt, int nbox, int axis, bool inverse,
                          cudaStream_t st, bool cb = false) {
  if (!c->gen) return launch_cols((int)c->N, box, bt, nbox, axis, inverse, c->d_tw, st);
  if (!box && nbox != bt.K) return cudaErrorInvalidValue;
  if (gen600_supported((int)c->N)) return launch_gen600_cols(box, bt, axis, inverse, cb, c->d_tw, st);
  return launch_gen_cols(c->gp, box, bt, axis, inverse, c->d_tw, st);
}
static cudaError_t x_cols_a_test(sf21_hii_ctx* c, const Batch& bt, cudaStream_t st) {
  if (c->gen && gen600_supported((int)c->N)) return launch_gen600_cols_a_test(bt, c->d_rc, c->d_alpha, c->d_tw, st);
  return c->gen ? launch_gen_cols_a_test(c->gp, bt, c->d_rc, c->d_alpha, c->d_tw, st)
                : launch_cols_a_test((int)c->N, bt, c->d_rc, c->d_alpha, c->d_tw, st);
}

// ---- schedule pieces --------------------------------------------------------
static int enqueue_front(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src,
                         cudaStream_t st) {
  int rc = prologue_args(c, z, kind, &c->pa);
  if (rc) return rc;
  float2* packed = c->d_work[0];
  const int N = (int)c->N;
  Batch none;
  memset(&none, 0, sizeof(none));
  int e0 = mark(c, st);
  CTX_CUDA(c, launch_prologue(c->n3, delta, src, c->pa, c->d_rec0, c->d_fres, packed, c->d_partials,
                              c->pro_blocks, st));
  int e1 = mark(c, st);
  CTX_CUDA(c, launch_alpha(c->d_partials, c->pro_blocks, c->d_alpha, st));
  int e2 = mark(c, st);
  CTX_CUDA(c, x_fwd_rows(c, packed, c->d_spec, c->d_alpha, st));
  int e3 = mark(c, st);
  CTX_CUDA(c, x_cols(c, c->d_spec, none, 1, 1, false, st));
  int e4 = mark(c, st);
  CTX_CUDA(c, x_cols(c, c->d_spec, none, 1, 0, false, st));
  int e5 = mark(c, st);
  CTX_CUDA(c, launch_finish_prep(c->n3, src, c->d_fres, c->pa, c->d_chain, c->d_om, st));
  int e6 = mark(c, st);
  span(c, KD_PREP, e5, e6);
  span(c, KD_PRO, e0, e1);
  span(c, KD_ALPHA, e1, e2);
  span(c, KD_FROWS, e2, e3);
  span(c, KD_FCB, e3, e4);
  span(c, KD_FCA, e4, e5);
  return SF21_OK;
}

// The radius pipeline of one batch: filter + inverse transform + centre test.
static int enqueue_batch(sf21_hii_ctx* c, const Batch& bt, cudaStream_t st) {
  const int N = (int)c->N;
  if (c->path == 2) {
    int e0 = mark(c, st);
    CTX_CUDA(c, launch_plane_filter(N, c->d_spec, bt, c->d_tw, st));
    int e1 = mark(c, st);
    CTX_CUDA(c, x_cols_a_test(c, bt, st));
    int e2 = mark(c, st);
    span(c, KD_PLANE, e0, e1);
    span(c, KD_ICA, e1, e2);
    return SF21_OK;
  }
  if (c->path == 8) {  // column-block-major work boxes, ky and kx in one launch
    int e0 = mark(c, st);
    CTX_CUDA(c, launch_rows_filter_cb(N, c->d_spec, bt, c->d_tw, st));
    int e1 = mark(c, st);
    CTX_CUDA(c, launch_cols_ba_fused(N, bt, c->d_rc32, c->d_alpha, c->d_tw, c->d_ctl, c->d_err, c->nsm, st,
                                     c->wait_limit));
    int e2 = mark(c, st);
    span(c, KD_IROWS, e0, e1);
    span(c, KD_FUSED, e1, e2);
    return SF21_OK;
  }
  if (c->path >= 5) {  // column-block-major work boxes
    int e0 = mark(c, st);
    CTX_CUDA(c, launch_rows_filter_cb(N, c->d_spec, bt, c->d_tw, st));
    int e1 = mark(c, st);
    if (c->path == 5)
      CTX_CUDA(c, launch_cols_b_cb(N, bt, c->d_tw, st));
    else
      CTX_CUDA(c, launch_pipe(N, 0, 1, c->pmaps, bt, c->d_work_base, c->d_rc, c->d_alpha, c->d_tw, c->d_err,
                              c->nsm, st, c->wait_limit));
    int e2 = mark(c, st);
    if (c->path == 7)
      CTX_CUDA(c, launch_pipe(N, 1, 1, c->pmaps, bt, c->d_work_base, c->d_rc, c->d_alpha, c->d_tw, c->d_err,
                              c->nsm, st, c->wait_limit));
    else
      CTX_CUDA(c, launch_cols_a_test_cb(N, bt, c->d_rc, c->d_alpha, c->d_tw, c->nsm, st));
    int e3 = mark(c, st);
    span(c, KD_IROWS, e0, e1);
    span(c, KD_ICB, e1, e2);
    span(c, KD_ICA, e2, e3);
    return SF21_OK;
  }
  if (c->path == 3 || c->path == 4) {
    int e0 = mark(c, st);
    CTX_CUDA(c, x_inv_rows_filter(c, c->d_spec, bt, st));
    int e1 = mark(c, st);
    CTX_CUDA(c, launch_pipe(N, 0, 0, c->pmaps, bt, c->d_work_base, c->d_rc, c->d_alpha, c->d_tw, c->d_err, c->nsm,
                            st, c->wait_limit));
    int e2 = mark(c, st);
    if (c->path == 4)
      CTX_CUDA(c, launch_pipe(N, 1, 0, c->pmaps, bt, c->d_work_base, c->d_rc, c->d_alpha, c->d_tw, c->d_err,
                              c->nsm, st, c->wait_limit));
    else
      CTX_CUDA(c, x_cols_a_test(c, bt, st));
    int e3 = mark(c, st);
    span(c, KD_IROWS, e0, e1);
    span(c, KD_ICB, e1, e2);
    span(c, KD_ICA, e2, e3);
    return SF21_OK;
  }
  // at N = 600 the batch's boxes are column-block major (the a-axis test pass reads them so)
  const bool cb600 = c->gen && gen600_supported(N);
  int e0 = mark(c, st);
  CTX_CUDA(c, x_inv_rows_filter(c, c->d_spec, bt, st, cb600));
  int e1 = mark(c, st);
  CTX_CUDA(c, x_cols(c, nullptr, bt, bt.K, 1, true, st, cb600));
  int e2 = mark(c, st);
  CTX_CUDA(c, x_cols_a_test(c, bt, st));
  int e3 = mark(c, st);
  span(c, KD_IROWS, e0, e1);
  span(c, KD_ICB, e1, e2);
  span(c, KD_ICA, e2, e3);
  return SF21_OK;
}

static int enqueue_radii(sf21_hii_ctx* c, int set, cudaStream_t st) {
  const SetInfo& s = c->sets[set];
  int rc;
  CTX_CUDA(c, cudaMemsetAsync(c->d_rc, RC_NONE, c->n3, st));
  if (c->path == 8) CTX_CUDA(c, cudaMemsetAsync(c->d_rc32, 0xFF, sizeof(unsigned int) * c->n3, st));
  const int nr = (int)s.R.size();
  for (int k0 = 0; k0 < nr; k0 += c->K) {
    Batch bt;
    memset(&bt, 0, sizeof(bt));
    bt.K = nr - k0 < c->K ? nr - k0 : c->K;
    bt.set = set;
    bt.zmul = (float)s.fesc;
    for (int k = 0; k < bt.K; ++k) {
      bt.r[k].dkR = (float)(c->dk * s.R[k0 + k]);
      bt.r[k].ridx = k0 + k;
      bt.r[k].work = c->d_work[k];
    }
    if ((rc = enqueue_batch(c, bt, st))) return rc;
  }
  if (c->path == 8) CTX_CUDA(c, launch_rc32_to_rc(c->n3, c->d_rc32, c->d_rc, st));
  return SF21_OK;
}

// Dilation + finish of one set; the per-voxel inputs (rec0, chain, om) are
// those of the last enqueue_front.
static int enqueue_finish(sf21_hii_ctx* c, int set, float* xhii, cudaStream_t st) {
  const SetInfo& s = c->sets[set];
  const int N = (int)c->N;
  int* dt0 = reinterpret_cast<int*>(c->d_work[0]);
  int* dt1 = dt0 + c->n3;
  int e0 = mark(c, st);
  CTX_CUDA(c, launch_dt_pa(N, c->d_rc, s.d_nmax, dt0, st));
  int e1 = mark(c, st);
  CTX_CUDA(c, launch_dt_pb(N, dt0, dt1, st));
  int e2 = mark(c, st);
  CTX_CUDA(c, launch_dt_pc_finish(N, dt1, dbits(s.fesc), c->d_chain, c->d_rec0, c->d_om, xhii, st));
  int e3 = mark(c, st);
  span(c, KD_DTR, e0, e1);
  span(c, KD_DTB, e1, e2);
  span(c, KD_DTA, e2, e3);
  return SF21_OK;
}

static int check_run_args(sf21_hii_ctx* c, int kind, const void* delta, const void* src, const void* out) {
  if (!c) return SF21_E_ARG;
  if (!delta || !src || !out) CTX_FAIL(c, SF21_E_ARG, "null buffer");
  if (kind != SF21_SRC_SFRD && kind != SF21_SRC_RION) CTX_FAIL(c, SF21_E_ARG, "unknown src_kind %d", kind);
  return SF21_OK;
}

static int enqueue_run(sf21_hii_ctx* c, double z, int kind, const float* delta_dev, const float* src_dev,
                       float* xhii_dev, cudaStream_t st) {
  int rc;
  if ((rc = enqueue_front(c, z, kind, delta_dev, src_dev, st))) return rc;
  for (int s = 0; s < (int)c->sets.size(); ++s) {
    if ((rc = enqueue_radii(c, s, st))) return rc;
    if ((rc = enqueue_finish(c, s, xhii_dev + (size_t)s * c->n3, st))) return rc;
  }
  return SF21_OK;
}

extern "C" int sf21_hii_run_z_device(sf21_hii_ctx* c, double z, int kind, const float* delta_dev,
                                     const float* src_dev, float* xhii_dev, void* stream) {
  int rc = check_run_args(c, kind, delta_dev, src_dev, xhii_dev);
  if (rc) return rc;
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  if (!c->use_graph || c->prof) return enqueue_run(c, z, kind, delta_dev, src_dev, xhii_dev, st);
  // replay the captured schedule if nothing it depends on changed
  sf21_hii_ctx::GraphKey key = {z, kind, delta_dev, src_dev, xhii_dev, st};
  const bool same = c->gexec && key.z == c->gkey.z && key.kind == c->gkey.kind && key.delta == c->gkey.delta &&
                    key.src == c->gkey.src && key.xhii == c->gkey.xhii && key.st == c->gkey.st;
  if (!same) {
    cudaGraph_t g = nullptr;
    CTX_CUDA(c, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_run(c, z, kind, delta_dev, src_dev, xhii_dev, st);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) CTX_FAIL(c, SF21_E_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
    bool updated = false;
    if (c->gexec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(c->gexec, g, &info) == cudaSuccess) {
        updated = true;
      } else {
        cudaGetLastError();
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
      }
    }
    if (!updated) {
      ce = cudaGraphInstantiate(&c->gexec, g, 0);
      if (ce != cudaSuccess) {
        cudaGraphDestroy(g);
        c->gexec = nullptr;
        CTX_FAIL(c, SF21_E_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ce));
      }
    }
    cudaGraphDestroy(g);
    c->gkey = key;
  }
  CTX_CUDA(c, cudaGraphLaunch(c->gexec, st));
  return SF21_OK;
}

// Radius loops and finish of every set, with each xHII box downloaded to
// the host while the GPU works on the next set: set s is written into
// staging box s mod 2 on the compute stream, copied out on the copy stream,
// and the staging box is reused only after its copy has completed.  Each
// set's neutral fraction is the serial double sum of the reference
// (:473-477), on a host thread once the box has arrived.
static int run_sets_to_host(sf21_hii_ctx* c, cudaStream_t st, float* xhii, double* neutral) {
  const size_t bf = sizeof(float) * c->n3;
  if (!c->copy_stream) {
    CTX_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
      CTX_CUDA(c, cudaEventCreateWithFlags(&c->ev_done[i], cudaEventDisableTiming));
      CTX_CUDA(c, cudaEventCreateWithFlags(&c->ev_copied[i], cudaEventDisableTiming));
    }
  }
  if (!c->d_xhii2) CTX_CUDA(c, dev_malloc(&c->d_xhii2, bf));
  float* stage[2] = {c->d_xhii, c->d_xhii2};
  std::vector<std::thread> sums;
  int status = SF21_OK;
  const int ns = (int)c->sets.size();
  auto start_sum = [&](int s) {
    if (!neutral) return;
    const float* dst = xhii + (size_t)s * c->n3;
    const long n3 = c->n3;
    double* out = neutral + s;
    sums.emplace_back([dst, n3, out]() {
      double acc = 0.;
      for (long i = 0; i < n3; ++i) acc += 1.0 - dst[i];
      *out = acc / n3;
    });
  };
  int copied = 0;  // sets whose download has been waited for
  for (int s = 0; s < ns && status == SF21_OK; ++s) {
    const int b = s & 1;
    cudaError_t e = cudaSuccess;
    if (s >= 2) e = cudaStreamWaitEvent(st, c->ev_copied[b], 0);  // staging box free again
    if (e == cudaSuccess && (status = enqueue_radii(c, s, st)) == SF21_OK &&
        (status = enqueue_finish(c, s, stage[b], st)) == SF21_OK) {
      e = cudaEventRecord(c->ev_done[b], st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->ev_done[b], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(xhii + (size_t)s * c->n3, stage[b], bf, cudaMemcpyDeviceToHost, c->copy_stream);
      if (e == cudaSuccess) e = cudaEventRecord(c->ev_copied[b], c->copy_stream);
      // the previous set's box has been on its way while this set was enqueued
      if (e == cudaSuccess && s >= 1) {
        e = cudaEventSynchronize(c->ev_copied[(s - 1) & 1]);
        if (e == cudaSuccess) start_sum(copied++);
      }
    }
    if (e != cudaSuccess) {
      c->err = std::string("xHII download failed: ") + cudaGetErrorString(e);
      status = SF21_E_CUDA;
    }
  }
  if (status == SF21_OK && copied < ns) {
    cudaError_t e = cudaEventSynchronize(c->ev_copied[(ns - 1) & 1]);
    if (e == cudaSuccess) {
      start_sum(copied++);
    } else {
      c->err = std::string("xHII download failed: ") + cudaGetErrorString(e);
      status = SF21_E_CUDA;
    }
  }
  cudaStreamSynchronize(c->copy_stream);
  for (std::thread& t : sums) t.join();
  if (status == SF21_OK) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      c->err = std::string("stream failed: ") + cudaGetErrorString(e);
      status = SF21_E_CUDA;
    }
  }
  if (status == SF21_OK) status = check_device_flag(c);
  return status;
}

extern "C" int sf21_hii_run_z(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src,
                              float* xhii, double* neutral) {
  int rc = check_run_args(c, kind, delta, src, xhii);
  if (rc) return rc;
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  const size_t bf = sizeof(float) * c->n3;
  CTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, bf, cudaMemcpyHostToDevice, st));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_src, src, bf, cudaMemcpyHostToDevice, st));
  if ((rc = enqueue_front(c, z, kind, c->d_delta, c->d_src, st))) return rc;
  return run_sets_to_host(c, st, xhii, neutral);
}

// ---- check hooks -------------------------------------------------------------
static int upload_front(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src) {
  int rc = check_run_args(c, kind, delta, src, delta);
  if (rc) return rc;
  CTX_CUDA(c, cudaSetDevice(c->device));
  const size_t bf = sizeof(float) * c->n3;
  CTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, bf, cudaMemcpyHostToDevice, c->stream));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_src, src, bf, cudaMemcpyHostToDevice, c->stream));
  return enqueue_front(c, z, kind, c->d_delta, c->d_src, c->stream);
}

extern "C" int sf21_hii_prologue(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src,
                                 int set, float* rec0, float* fresid, float* fill0) {
  if (!c || set < 0 || set >= (int)c->sets.size()) return SF21_E_ARG;
  int rc = upload_front(c, z, kind, delta, src);
  if (rc) return rc;
  const size_t bf = sizeof(float) * c->n3;
  CTX_CUDA(c, launch_fill0(c->n3, dbits(c->sets[set].fesc), c->d_src, c->d_rec0, c->pa, c->d_xhii, c->stream));
  if (rec0) CTX_CUDA(c, cudaMemcpyAsync(rec0, c->d_rec0, bf, cudaMemcpyDeviceToHost, c->stream));
  if (fresid) CTX_CUDA(c, cudaMemcpyAsync(fresid, c->d_fres, bf, cudaMemcpyDeviceToHost, c->stream));
  if (fill0) CTX_CUDA(c, cudaMemcpyAsync(fill0, c->d_xhii, bf, cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

extern "C" int sf21_hii_filtered(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src,
                                 int set, int ridx, float* rec_R, float* ion_R) {
  if (!c || set < 0 || set >= (int)c->sets.size()) return SF21_E_ARG;
  const SetInfo& s = c->sets[set];
  if (ridx < 0 || ridx >= (int)s.R.size() || !rec_R || !ion_R) CTX_FAIL(c, SF21_E_ARG, "bad radius index");
  int rc = upload_front(c, z, kind, delta, src);
  if (rc) return rc;
  // filtered inverse transform of one radius, without the centre test
  Batch bt;
  memset(&bt, 0, sizeof(bt));
  bt.K = 1;
  bt.zmul = (float)s.fesc;
  bt.r[0].dkR = (float)(c->dk * s.R[ridx]);
  bt.r[0].ridx = ridx;
  bt.r[0].work = c->d_work[0];
  const int N = (int)c->N;
  CTX_CUDA(c, x_inv_rows_filter(c, c->d_spec, bt, c->stream));
  CTX_CUDA(c, x_cols(c, c->d_work[0], bt, 1, 1, true, c->stream));
  CTX_CUDA(c, x_cols(c, c->d_work[0], bt, 1, 0, true, c->stream));
  std::vector<float2> box(c->n3);
  float alpha = 1.f;
  CTX_CUDA(c, cudaMemcpyAsync(box.data(), c->d_work[0], sizeof(float2) * c->n3, cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaMemcpyAsync(&alpha, c->d_alpha, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  for (long i = 0; i < c->n3; ++i) {
    rec_R[i] = box[i].x;
    ion_R[i] = alpha > 0.f ? (float)((double)box[i].y * s.fesc / alpha) : 0.0f;  // alpha < 0: no source
  }
  return SF21_OK;
}

extern "C" int sf21_hii_first_hit(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src,
                                  int set, uint8_t* rcout) {
  if (!c || set < 0 || set >= (int)c->sets.size() || !rcout) return SF21_E_ARG;
  int rc = upload_front(c, z, kind, delta, src);
  if (rc) return rc;
  if ((rc = enqueue_radii(c, set, c->stream))) return rc;
  CTX_CUDA(c, cudaMemcpyAsync(rcout, c->d_rc, c->n3, cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

// ---- measurement hooks ---------------------------------------------------------
extern "C" int sf21_hii_profile(sf21_hii_ctx* c, int enable) {
  if (!c) return SF21_E_ARG;
  c->prof = enable != 0;
  c->ev_used = 0;
  c->spans.clear();
  for (int k = 0; k < KD_COUNT; ++k) {
    c->prof_ms[k] = 0;
    c->prof_n[k] = 0;
  }
  return SF21_OK;
}

extern "C" int sf21_hii_profile_read(sf21_hii_ctx* c, double* ms, long* launches, int cap) {
  if (!c) return SF21_E_ARG;
  CTX_CUDA(c, cudaSetDevice(c->device));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  if (!c->spans.empty()) CTX_CUDA(c, cudaEventSynchronize(c->ev[c->spans.back().b]));
  for (const auto& sp : c->spans) {
    float t = 0.f;
    CTX_CUDA(c, cudaEventElapsedTime(&t, c->ev[sp.a], c->ev[sp.b]));
    c->prof_ms[sp.kind] += t;
    c->prof_n[sp.kind] += 1;
  }
  c->spans.clear();
  c->ev_used = 0;
  for (int k = 0; k < KD_COUNT && k < cap; ++k) {
    if (ms) ms[k] = c->prof_ms[k];
    if (launches) launches[k] = c->prof_n[k];
  }
  return KD_COUNT;
}

extern "C" const char* sf21_hii_profile_name(int kind) {
  return (kind >= 0 && kind < KD_COUNT) ? kKindNames[kind] : "";
}

// ---- plain form: one radius per launch sequence, reference structure ----------
extern "C" int sf21_hii_run_z_plain_device(sf21_hii_ctx* c, double z, int kind, const float* delta_dev,
                                           const float* src_dev, int set, float* xhii_dev, void* stream) {
  int rc = check_run_args(c, kind, delta_dev, src_dev, xhii_dev);
  if (rc) return rc;
  if (set < 0 || set >= (int)c->sets.size()) CTX_FAIL(c, SF21_E_ARG, "bad set index %d", set);
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const int N = (int)c->N;
  const long n3 = c->n3;
  if (!c->d_mask) CTX_CUDA(c, dev_malloc(&c->d_mask, sizeof(float) * n3));
  if (!c->d_flag) CTX_CUDA(c, dev_malloc(&c->d_flag, sizeof(int)));
  if (!c->d_box2) CTX_CUDA(c, dev_malloc(&c->d_box2, sizeof(float2) * n3));
  if ((rc = enqueue_front(c, z, kind, delta_dev, src_dev, st))) return rc;
  const SetInfo& s = c->sets[set];
  // single-cell fill (:281-288) into the output box
  CTX_CUDA(c, launch_fill0(n3, dbits(s.fesc), src_dev, c->d_rec0, c->pa, xhii_dev, st));
  float2* box = c->d_work[0];
  Batch none;
  memset(&none, 0, sizeof(none));
  for (int i = 0; i < (int)s.R.size(); ++i) {
    Batch bt;
    memset(&bt, 0, sizeof(bt));
    bt.K = 1;
    bt.zmul = (float)s.fesc;
    bt.r[0].dkR = (float)(c->dk * s.R[i]);
    bt.r[0].ridx = i;
    bt.r[0].work = box;
    // filtered fields (:305-325)
    CTX_CUDA(c, x_inv_rows_filter(c, c->d_spec, bt, st));
    CTX_CUDA(c, x_cols(c, box, none, 1, 1, true, st));
    CTX_CUDA(c, x_cols(c, box, none, 1, 0, true, st));
    CTX_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), st));
    CTX_CUDA(c, launch_plain_centres(n3, box, c->d_alpha, (float)s.fesc, c->d_mask, c->d_flag, st));
    if (i < s.n_fft) {
      // FFT convolution with the discrete sphere (:358-393)
      CTX_CUDA(c, launch_plain_pack_sphere(N, s.nmax[i], c->d_mask, c->d_flag, c->d_box2, st));
      CTX_CUDA(c, x_fwd_rows(c, c->d_box2, c->d_box2, nullptr, st));
      CTX_CUDA(c, x_cols(c, c->d_box2, none, 1, 1, false, st));
      CTX_CUDA(c, x_cols(c, c->d_box2, none, 1, 0, false, st));
      CTX_CUDA(c, launch_plain_product(N, c->d_box2, c->d_flag, box, st));
      CTX_CUDA(c, x_inv_rows_plain(c, box, st));
      CTX_CUDA(c, x_cols(c, box, none, 1, 1, true, st));
      CTX_CUDA(c, x_cols(c, box, none, 1, 0, true, st));
      CTX_CUDA(c, launch_plain_threshold(n3, box, c->d_flag, xhii_dev, st));
    } else {
      // ball painting (:427-458)
      CTX_CUDA(c, launch_plain_paint(N, (int)(long)(s.R[i] / c->dx), s.nmax[i], c->d_mask, xhii_dev, st));
    }
  }
  CTX_CUDA(c, launch_plain_cap(n3, c->d_fres, xhii_dev, st));
  return SF21_OK;
}

extern "C" int sf21_hii_path(const sf21_hii_ctx* c, double* ms_tuned, int cap) {
  if (!c) return -SF21_E_ARG;
  for (int p = 1; p <= NPATH && p <= cap; ++p) ms_tuned[p - 1] = c->tune_ms[p] < 1e29 ? c->tune_ms[p] : 0.0;
  return c->path;
}

// Status of the bounded device waits: SF21_E_TIMEOUT if one expired since the
// last check (the flag is cleared), else SF21_OK.
static int check_device_flag(sf21_hii_ctx* c) {
  int f = 0;
  CTX_CUDA(c, cudaMemcpy(&f, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (f) {
    CTX_CUDA(c, cudaMemset(c->d_err, 0, sizeof(int)));
    CTX_FAIL(c, SF21_E_TIMEOUT, "a bounded device wait expired (TMA copy did not complete)");
  }
  return SF21_OK;
}

extern "C" int sf21_hii_inject_alloc_failure(long n) {
  if (n < 0) return SF21_E_ARG;
  sf21::g_fail_alloc_in.store(n);
  return SF21_OK;
}

extern "C" int sf21_hii_set_wait_limit(sf21_hii_ctx* c, unsigned int polls) {
  if (!c) return SF21_E_ARG;
  c->wait_limit = polls;
  // the captured graph holds the old limit in its kernel arguments
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  return SF21_OK;
}

extern "C" int sf21_hii_batch_radii(const sf21_hii_ctx* c) { return c ? c->K : -SF21_E_ARG; }

extern "C" int sf21_hii_check(sf21_hii_ctx* c) {
  if (!c) return SF21_E_ARG;
  CTX_CUDA(c, cudaSetDevice(c->device));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_device_flag(c);
}

// ---- criterion C(x) = max_R ion_R / rec_R and its vector-Jacobian product ----
static int ensure_adj_buffers(sf21_hii_ctx* c) {
  const long n3 = c->n3;
  if (!c->d_C) CTX_CUDA(c, dev_malloc(&c->d_C, sizeof(float) * n3));
  if (!c->d_A) CTX_CUDA(c, dev_malloc(&c->d_A, n3));
  return SF21_OK;
}

// recompute the filtered fields of a batch up to (not including) the kx pass
static int enqueue_recompute(sf21_hii_ctx* c, const Batch& bt, cudaStream_t st) {
  const int N = (int)c->N;
  if (c->path == 2) {
    int e0 = mark(c, st);
    CTX_CUDA(c, launch_plane_filter(N, c->d_spec, bt, c->d_tw, st));
    span(c, KD_PLANE, e0, mark(c, st));
  } else {
    int e0 = mark(c, st);
    CTX_CUDA(c, x_inv_rows_filter(c, c->d_spec, bt, st));
    int e1 = mark(c, st);
    CTX_CUDA(c, x_cols(c, nullptr, bt, bt.K, 1, true, st));
    span(c, KD_IROWS, e0, e1);
    span(c, KD_ICB, e1, mark(c, st));
  }
  return SF21_OK;
}

static Batch make_batch(const sf21_hii_ctx* c, int set, int k0, int nr) {
  const SetInfo& s = c->sets[set];
  Batch bt;
  memset(&bt, 0, sizeof(bt));
  bt.K = nr - k0 < c->K ? nr - k0 : c->K;
  bt.set = set;
  bt.zmul = (float)s.fesc;
  for (int k = 0; k < bt.K; ++k) {
    bt.r[k].dkR = (float)(c->dk * s.R[k0 + k]);
    bt.r[k].ridx = k0 + k;
    bt.r[k].work = c->d_work[k];
  }
  return bt;
}

extern "C" int sf21_hii_criterion_device(sf21_hii_ctx* c, double z, int kind, const float* delta_dev,
                                         const float* src_dev, int set, float* C_dev, uint8_t* argmax_dev,
                                         void* stream) {
  int rc = check_run_args(c, kind, delta_dev, src_dev, C_dev);
  if (rc) return rc;
  if (set < 0 || set >= (int)c->sets.size()) CTX_FAIL(c, SF21_E_ARG, "bad set index %d", set);
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  if ((rc = ensure_adj_buffers(c))) return rc;
  if ((rc = enqueue_front(c, z, kind, delta_dev, src_dev, st))) return rc;
  const int N = (int)c->N;
  CTX_CUDA(c, launch_crit_init(c->n3, c->d_C, c->d_A, st));
  const int nr = c->sets[set].n_fft;  // radii of the FFT branch (R >= 2 dx)
  for (int k0 = 0; k0 < nr; k0 += c->K) {
    Batch bt = make_batch(c, set, k0, nr);
    if ((rc = enqueue_recompute(c, bt, st))) return rc;
    int e0 = mark(c, st);
    if (c->gen) {  // shared-memory transforms: whole a-axis pass, then the per-element rule
      CTX_CUDA(c, x_cols(c, nullptr, bt, bt.K, 0, true, st));
      CTX_CUDA(c, launch_crit_elem(c->n3, bt, c->d_C, c->d_A, c->d_alpha, st));
    } else {
      CTX_CUDA(c, launch_cols_a_crit(N, bt, c->d_C, c->d_A, c->d_alpha, c->d_tw, st));
    }
    span(c, KD_CRIT, e0, mark(c, st));
  }
  CTX_CUDA(c, launch_crit_finalize(c->n3, c->d_C, c->d_A, st));
  if (C_dev != c->d_C)
    CTX_CUDA(c, cudaMemcpyAsync(C_dev, c->d_C, sizeof(float) * c->n3, cudaMemcpyDeviceToDevice, st));
  if (argmax_dev && argmax_dev != c->d_A)
    CTX_CUDA(c, cudaMemcpyAsync(argmax_dev, c->d_A, c->n3, cudaMemcpyDeviceToDevice, st));
  c->crit_set = set;
  c->crit_z = z;
  return SF21_OK;
}

extern "C" int sf21_hii_vjp_device(sf21_hii_ctx* c, double z, int kind, const float* delta_dev,
                                   const float* src_dev, int set, const float* dC_dev, float* ddelta_dev,
                                   float* dsrc_dev, double* dzeta, void* stream) {
  int rc = check_run_args(c, kind, delta_dev, src_dev, dC_dev);
  if (rc) return rc;
  if (set != c->crit_set || z != c->crit_z || !c->d_A)
    CTX_FAIL(c, SF21_E_ARG, "vjp needs the argmax checkpoint of a criterion call for the same set and z");
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const int N = (int)c->N;
  const long n3 = c->n3;
  const int nzp = c->gen ? adj_elem_blocks() : adj_zpart_blocks(N);
  if (!c->d_acc) CTX_CUDA(c, dev_malloc(&c->d_acc, sizeof(float2) * n3));
  if (!c->d_zpart) CTX_CUDA(c, dev_malloc(&c->d_zpart, sizeof(float) * nzp));
  // recompute the spectrum (the checkpoint holds only the argmax index)
  if ((rc = enqueue_front(c, z, kind, delta_dev, src_dev, st))) return rc;
  CTX_CUDA(c, cudaMemsetAsync(c->d_acc, 0, sizeof(float2) * n3, st));
  CTX_CUDA(c, cudaMemsetAsync(c->d_zpart, 0, sizeof(float) * nzp, st));
  Batch none;
  memset(&none, 0, sizeof(none));
  const int nr = c->sets[set].n_fft;
  for (int k0 = 0; k0 < nr; k0 += c->K) {
    Batch bt = make_batch(c, set, k0, nr);
    if ((rc = enqueue_recompute(c, bt, st))) return rc;
    int e0 = mark(c, st);
    if (c->gen) {  // a-axis inverse, cotangents, a-axis forward as whole-box passes
      CTX_CUDA(c, x_cols(c, nullptr, bt, bt.K, 0, true, st));
      CTX_CUDA(c, launch_adj_elem(n3, bt, dC_dev, c->d_A, c->d_alpha, c->d_zpart, st));
      CTX_CUDA(c, x_cols(c, nullptr, bt, bt.K, 0, false, st));
    } else {
      CTX_CUDA(c, launch_cols_a_adj(N, bt, dC_dev, c->d_A, c->d_alpha, c->d_zpart, c->d_tw, st));
    }
    int e1 = mark(c, st);
    CTX_CUDA(c, x_cols(c, nullptr, bt, bt.K, 1, false, st));
    int e2 = mark(c, st);
    if (c->gen) {  // c-axis forward of each box, then W and the sum over the batch
      for (int k = 0; k < bt.K; ++k)
        CTX_CUDA(c, x_fwd_rows(c, bt.r[k].work, bt.r[k].work, nullptr, st));
      CTX_CUDA(c, launch_acc_elem(N, bt, c->d_acc, st));
    } else {
      CTX_CUDA(c, launch_rows_adj_acc(N, bt, c->d_acc, c->d_tw, st));
    }
    int e3 = mark(c, st);
    span(c, KD_ADJA, e0, e1);
    span(c, KD_ADJB, e1, e2);
    span(c, KD_ADJR, e2, e3);
  }
  // back to real space: sum_R B_R (cotangents)
  int f0 = mark(c, st);
  CTX_CUDA(c, x_inv_rows_plain(c, c->d_acc, st));
  CTX_CUDA(c, x_cols(c, c->d_acc, none, 1, 1, true, st));
  CTX_CUDA(c, x_cols(c, c->d_acc, none, 1, 0, true, st));
  double mul = 1.0;
  for (int m = 0; m < c->pa.n_src_mul; ++m) {
    double v;
    memcpy(&v, &c->pa.src_mul[m], 8);
    mul *= v;
  }
  CTX_CUDA(c, launch_grad_finish(n3, c->d_acc, c->d_alpha, delta_dev, c->d_rec0, 1.76105133f, 0.81722878f,
                                 (float)mul, ddelta_dev, dsrc_dev, st));
  span(c, KD_ADJF, f0, mark(c, st));
  if (dzeta) {
    std::vector<float> zp(nzp);
    CTX_CUDA(c, cudaMemcpyAsync(zp.data(), c->d_zpart, sizeof(float) * nzp, cudaMemcpyDeviceToHost, st));
    CTX_CUDA(c, cudaStreamSynchronize(st));
    double s = 0.0;
    for (float v : zp) s += v;
    *dzeta = s;
  }
  return SF21_OK;
}

extern "C" int sf21_hii_criterion(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src,
                                  int set, float* C, uint8_t* argmax) {
  int rc = check_run_args(c, kind, delta, src, C);
  if (rc) return rc;
  CTX_CUDA(c, cudaSetDevice(c->device));
  const size_t bf = sizeof(float) * c->n3;
  CTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, bf, cudaMemcpyHostToDevice, c->stream));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_src, src, bf, cudaMemcpyHostToDevice, c->stream));
  if ((rc = ensure_adj_buffers(c))) return rc;
  if ((rc = sf21_hii_criterion_device(c, z, kind, c->d_delta, c->d_src, set, c->d_C, c->d_A, c->stream)))
    return rc;
  CTX_CUDA(c, cudaMemcpyAsync(C, c->d_C, bf, cudaMemcpyDeviceToHost, c->stream));
  if (argmax) CTX_CUDA(c, cudaMemcpyAsync(argmax, c->d_A, c->n3, cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

extern "C" int sf21_hii_vjp(sf21_hii_ctx* c, double z, int kind, const float* delta, const float* src, int set,
                            const float* dC, float* ddelta, float* dsrc, double* dzeta) {
  int rc = check_run_args(c, kind, delta, src, dC);
  if (rc) return rc;
  CTX_CUDA(c, cudaSetDevice(c->device));
  const size_t bf = sizeof(float) * c->n3;
  if (!c->d_g) CTX_CUDA(c, dev_malloc(&c->d_g, bf));
  if (ddelta && !c->d_gd) CTX_CUDA(c, dev_malloc(&c->d_gd, bf));
  if (dsrc && !c->d_gs) CTX_CUDA(c, dev_malloc(&c->d_gs, bf));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, bf, cudaMemcpyHostToDevice, c->stream));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_src, src, bf, cudaMemcpyHostToDevice, c->stream));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_g, dC, bf, cudaMemcpyHostToDevice, c->stream));
  if ((rc = sf21_hii_vjp_device(c, z, kind, c->d_delta, c->d_src, set, c->d_g, ddelta ? c->d_gd : nullptr,
                                dsrc ? c->d_gs : nullptr, dzeta, c->stream)))
    return rc;
  if (ddelta) CTX_CUDA(c, cudaMemcpyAsync(ddelta, c->d_gd, bf, cudaMemcpyDeviceToHost, c->stream));
  if (dsrc) CTX_CUDA(c, cudaMemcpyAsync(dsrc, c->d_gs, bf, cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

// ---- halo-catalogue source box on the GPU ---------------------------------------
static int enqueue_halo_source(sf21_hii_ctx* c, double z, long nhalos, const void* halos, float* out_dev,
                               cudaStream_t st) {
  if (nhalos < 0 || (nhalos > 0 && !halos)) CTX_FAIL(c, SF21_E_ARG, "bad halo catalogue");
  if (c->N_halo < c->N) CTX_FAIL(c, SF21_E_ARG, "N_halo < N_smoothed (smooth_box, auxiliary.c:651-654)");
  if (nhalos >= (1L << 28)) CTX_FAIL(c, SF21_E_UNSUPPORTED, "2^28 halos or more (8 CIC entries each, int count)");
  const long nh3 = c->N_halo * c->N_halo * c->N_halo;
  if (!c->d_fine) CTX_CUDA(c, dev_malloc(&c->d_fine, sizeof(float) * nh3));
  if (nhalos > c->halo_cap) {
    if (c->d_halos) cudaFree(c->d_halos);
    if (c->d_hscratch) cudaFree(c->d_hscratch);
    c->d_halos = nullptr;
    c->d_hscratch = nullptr;
    c->halo_cap = 0;
    const long cap = nhalos + nhalos / 4 + 1024;
    CTX_CUDA(c, dev_malloc(&c->d_halos, (size_t)cap * 16));
    c->hscratch_bytes = halo_scratch_bytes(cap);
    CTX_CUDA(c, dev_malloc(&c->d_hscratch, c->hscratch_bytes));
    c->halo_cap = cap;
  }
  if (nhalos > 0)
    CTX_CUDA(c, cudaMemcpyAsync(c->d_halos, halos, (size_t)nhalos * 16, cudaMemcpyHostToDevice, st));
  CTX_CUDA(c, launch_halo_source(nhalos, c->d_halos, z, c->N_halo, c->N, c->d_fine, out_dev, c->d_hscratch,
                                 c->hscratch_bytes, st));
  return SF21_OK;
}

extern "C" int sf21_hii_halo_source(sf21_hii_ctx* c, double z, long nhalos, const void* halos, float* rion) {
  if (!c || !rion) return SF21_E_ARG;
  CTX_CUDA(c, cudaSetDevice(c->device));
  int rc = enqueue_halo_source(c, z, nhalos, halos, c->d_src, c->stream);
  if (rc) return rc;
  CTX_CUDA(c, cudaMemcpyAsync(rion, c->d_src, sizeof(float) * c->n3, cudaMemcpyDeviceToHost, c->stream));
  CTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

extern "C" int sf21_hii_run_z_halos(sf21_hii_ctx* c, double z, const float* delta, long nhalos, const void* halos,
                                    float* xhii, double* neutral) {
  if (!c || !delta || !xhii) return SF21_E_ARG;
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  const size_t bf = sizeof(float) * c->n3;
  int rc = enqueue_halo_source(c, z, nhalos, halos, c->d_src, st);
  if (rc) return rc;
  CTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, bf, cudaMemcpyHostToDevice, st));
  if ((rc = enqueue_front(c, z, SF21_SRC_RION, c->d_delta, c->d_src, st))) return rc;
  return run_sets_to_host(c, st, xhii, neutral);
}

// ---- power spectrum (tools/power3d_f.c:124-194) -------------------------------
// Window factor per axis, the reference's wind() (power3d_f.c:205-211).
static double pk_axis_window(int x, int n, int flag) {
  const double m = (double)(n - 1);
  if (flag == 1) return 1 - fabs(x - m / 2.) / m * 2.;
  if (flag == 2) return 1 - ((x - m / 2.) / m * 2.) * ((x - m / 2.) / m * 2.);
  return 1.0;
}

static int power_spectrum_device(sf21_hii_ctx* c, const float* box_dev, int flag, double dl, double* k, double* P,
                                 int cap, cudaStream_t st, int* nk_out) {
  if (!box_dev || !(dl > 0) || flag < 0 || flag > 2 || cap < 0 || (cap > 0 && (!k || !P)))
    CTX_FAIL(c, SF21_E_ARG, "power spectrum: bad arguments");
  const int N = (int)c->N;
  const int nk = pk_nbins(N);
  const int grid = pk_bin_grid(N);
  if (!c->d_pk) CTX_CUDA(c, dev_malloc(&c->d_pk, sizeof(float2) * c->n3));
  if (!c->d_pk_w) CTX_CUDA(c, dev_malloc(&c->d_pk_w, sizeof(float) * N));
  if (!c->d_pk_part) CTX_CUDA(c, dev_malloc(&c->d_pk_part, sizeof(float) * (size_t)grid * nk));
  if (!c->d_pk_cnt) CTX_CUDA(c, dev_malloc(&c->d_pk_cnt, sizeof(unsigned long long) * nk));
  std::vector<float> wax(N);
  double s1 = 0.;
  for (int x = 0; x < N; ++x) {
    const double w = pk_axis_window(x, N, flag);
    wax[x] = (float)w;
    s1 += w * w;
  }
  const double wsum = s1 * s1 * s1;  // the window is separable: sum of its square = product of the axis sums
  float2* packed = c->d_work[0];
  Batch none;
  memset(&none, 0, sizeof(none));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_pk_w, wax.data(), sizeof(float) * N, cudaMemcpyHostToDevice, st));
  CTX_CUDA(c, launch_pk_pack(N, box_dev, c->d_pk_w, packed, st));
  CTX_CUDA(c, x_fwd_rows(c, packed, c->d_pk, nullptr, st));
  CTX_CUDA(c, x_cols(c, c->d_pk, none, 1, 1, false, st));
  CTX_CUDA(c, x_cols(c, c->d_pk, none, 1, 0, false, st));
  CTX_CUDA(c, cudaMemsetAsync(c->d_pk_cnt, 0, sizeof(unsigned long long) * nk, st));
  CTX_CUDA(c, launch_pk_bin(N, c->d_pk, nk, c->d_pk_part, c->d_pk_cnt, st));
  std::vector<float> part((size_t)grid * nk);
  std::vector<unsigned long long> cnt(nk);
  CTX_CUDA(c, cudaMemcpyAsync(part.data(), c->d_pk_part, sizeof(float) * part.size(), cudaMemcpyDeviceToHost, st));
  CTX_CUDA(c, cudaMemcpyAsync(cnt.data(), c->d_pk_cnt, sizeof(unsigned long long) * nk, cudaMemcpyDeviceToHost, st));
  CTX_CUDA(c, cudaStreamSynchronize(st));
  const double dk = 2.0 * kPI / (N * dl);
  const double dl3 = dl * dl * dl;
  for (int b = 0; b < nk && b < cap; ++b) {
    double sum = 0.;
    for (int g = 0; g < grid; ++g) sum += (double)part[(size_t)g * nk + b];
    const double n = cnt[b] ? (double)cnt[b] : 1.0;
    k[b] = b * dk;
    P[b] = sum / n / wsum * dl3;
  }
  *nk_out = nk;
  return SF21_OK;
}

extern "C" int sf21_hii_power_spectrum_device(sf21_hii_ctx* c, const float* box_dev, int flag, double dl, double* k,
                                              double* P, int cap, void* stream) {
  if (!c) return -SF21_E_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return -SF21_E_CUDA;
  int nk = 0;
  const int rc =
      power_spectrum_device(c, box_dev, flag, dl, k, P, cap, stream ? (cudaStream_t)stream : c->stream, &nk);
  return rc ? -rc : nk;  // nk >= 1, or minus a status code
}

extern "C" int sf21_hii_power_spectrum(sf21_hii_ctx* c, const float* box, int flag, double dl, double* k, double* P,
                                       int cap) {
  if (!c || !box) return -SF21_E_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return -SF21_E_CUDA;
  if (cudaMemcpyAsync(c->d_delta, box, sizeof(float) * c->n3, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
    c->err = "power spectrum: box upload failed";
    return -SF21_E_CUDA;
  }
  int nk = 0;
  const int rc = power_spectrum_device(c, c->d_delta, flag, dl, k, P, cap, c->stream, &nk);
  return rc ? -rc : nk;
}

// ---- 21-cm brightness temperature (t21.c:114-255) ----------------------------
namespace {
constexpr double kH0 = 3.24078e-18;  // h/sec, Input_variables.h:108
constexpr double kTcmb0 = 2.725;     // K, t21.c:25
struct T21Cosmo {
  double om, ob, ol, h;
  double Hz(double z) const { return h * kH0 * sqrt(om * (1. + z) * (1. + z) * (1. + z) + ol); }  // auxiliary.c:224
  double int_growth(double zz) const {  // auxiliary.c:243-257
    const double dz = 0.001;
    double intg = 0., z;
    const double hz0 = Hz(0.);
    for (z = zz + dz / 2.; z < zz + 100.; z += dz) {
      const double hub = Hz(z) / hz0;
      intg += (1. + z) / hub / hub / hub;
    }
    return intg * dz;
  }
  double growth(double z) const { return Hz(z) / Hz(0) * int_growth(z) / int_growth(0.); }  // :262-266
  double dgrowth_dt(double z) const {  // :285-291, dz/dt = -H(z) (1 + z)
    const double dz = 1e-3;
    return (growth(z + dz / 2.) - growth(z - dz / 2.)) / dz * (-Hz(z) * (1.0 + z));
  }
};
}  // namespace

extern "C" int sf21_t21_run_z(sf21_hii_ctx* c, const sf21_t21_cosmo* cosmo, double z, const float* delta,
                              const float* xhii, const float* xc, const float* xalpha, const float* tempx,
                              float* tb, double* tb_mean, double* ts_mean) {
  if (!c) return SF21_E_ARG;
  if (!cosmo || !delta || !xhii || !tb) CTX_FAIL(c, SF21_E_ARG, "t21: null argument");
  const bool spin = xc != nullptr;
  if (spin != (xalpha != nullptr) || spin != (tempx != nullptr))
    CTX_FAIL(c, SF21_E_ARG, "t21: xc, xalpha and tempx must be all given or all NULL");
  CTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  const long n3 = c->n3;
  const int N = (int)c->N;
  const size_t bf = sizeof(float) * n3;
  const int nb = t21_blocks(n3);
  if (!c->d_pk) CTX_CUDA(c, dev_malloc(&c->d_pk, sizeof(float2) * n3));
  if (!c->d_t21) CTX_CUDA(c, dev_malloc(&c->d_t21, 4 * bf));
  if (!c->d_t21_part) CTX_CUDA(c, dev_malloc(&c->d_t21_part, sizeof(float) * 2 * nb));
  float* d_xc = c->d_t21;
  float* d_xa = d_xc + n3;
  float* d_tk = d_xa + n3;
  float* d_tb = d_tk + n3;
  CTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, bf, cudaMemcpyHostToDevice, st));
  CTX_CUDA(c, cudaMemcpyAsync(c->d_xhii, xhii, bf, cudaMemcpyHostToDevice, st));
  if (spin) {
    CTX_CUDA(c, cudaMemcpyAsync(d_xc, xc, bf, cudaMemcpyHostToDevice, st));
    CTX_CUDA(c, cudaMemcpyAsync(d_xa, xalpha, bf, cudaMemcpyHostToDevice, st));
    CTX_CUDA(c, cudaMemcpyAsync(d_tk, tempx, bf, cudaMemcpyHostToDevice, st));
  }
  // scalars in double on the host, as the reference
  const T21Cosmo cs{cosmo->omega_m, cosmo->omega_b, cosmo->omega_lambda, c->hubble};
  const double L = c->L, dx = c->dx, h = c->hubble;
  T21Args ta;
  ta.scale = (float)(-cs.dgrowth_dt(z) / L / L / L / cs.Hz(z) * dx * dx * dx / cs.growth(z));
  ta.pref = (float)(23.0 / 1000. * (0.7 / h) * (cs.ob * h * h / 0.02) * sqrt((0.15 / cs.om / h / h) * (1. + z) / 10.));
  ta.tcmb = (float)(kTcmb0 * (1. + z));
  Batch none;
  memset(&none, 0, sizeof(none));
  float2* packed = c->d_work[0];
  CTX_CUDA(c, launch_t21_pack(n3, c->d_delta, packed, st));
  CTX_CUDA(c, x_fwd_rows(c, packed, c->d_pk, nullptr, st));
  CTX_CUDA(c, x_cols(c, c->d_pk, none, 1, 1, false, st));
  CTX_CUDA(c, x_cols(c, c->d_pk, none, 1, 0, false, st));
  CTX_CUDA(c, launch_t21_kfilter(N, cosmo->vel_comp, c->d_pk, st));
  CTX_CUDA(c, x_inv_rows_plain(c, c->d_pk, st));
  CTX_CUDA(c, x_cols(c, c->d_pk, none, 1, 1, true, st));
  CTX_CUDA(c, x_cols(c, c->d_pk, none, 1, 0, true, st));
  CTX_CUDA(c, launch_t21_finish(n3, c->d_pk, c->d_delta, c->d_xhii, spin ? d_xc : nullptr, spin ? d_xa : nullptr,
                                spin ? d_tk : nullptr, ta, d_tb, c->d_t21_part, st));
  std::vector<float> part(2 * (size_t)nb);
  CTX_CUDA(c, cudaMemcpyAsync(tb, d_tb, bf, cudaMemcpyDeviceToHost, st));
  CTX_CUDA(c, cudaMemcpyAsync(part.data(), c->d_t21_part, sizeof(float) * part.size(), cudaMemcpyDeviceToHost, st));
  CTX_CUDA(c, cudaStreamSynchronize(st));
  double s_tb = 0., s_ts = 0.;
  for (int b = 0; b < nb; ++b) {
    s_tb += part[2 * b];
    s_ts += part[2 * b + 1];
  }
  if (tb_mean) *tb_mean = s_tb / n3;
  if (ts_mean) *ts_mean = spin ? s_ts / n3 : 0.0;
  return SF21_OK;
}
