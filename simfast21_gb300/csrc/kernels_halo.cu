// Halo-catalogue source box on the GPU (use_SFR = F branch of the stage,
// get_HIIbubbles.c:229-253): Rion(M, z) of every halo (user_functions.c:40-47),
// cloud-in-cell deposit on the N_halo^3 grid (auxiliary.c:761-808) and the
// block average to N_smooth^3 (auxiliary.c:643-684) -- bit-identical with the
// reference's serial loop.  The star-formation-rate stage (get_SFR.c:114-131)
// is the same deposit with the weight sfr(M, z) = Rion(M, z) / Qion(z)
// (user_functions.c:71-75) and each smoothed cell divided by dx_halo^3.
//
// The reference adds the 8 CIC contributions of halo 0, then halo 1, ... into
// a float box (float += double each time), so a cell's value depends on the
// order of its contributions.  Here every contribution is computed in
// parallel (same float/double steps, integer soft-double for the double
// ones), tagged with its serial position, grouped by cell with a stable radix
// sort (the serial order survives inside each cell), and each cell's chain is
// replayed in that order.  The block average repeats the reference's double
// sum in its loop order.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/sf21_hii.h"

#include "sf21_kernels.h"
#include "softdouble.h"

namespace sf21 {

struct HaloRec {  // Halo_t, auxiliary.h:13-17
  float Mass, x, y, z;
};

__device__ __forceinline__ long wrap_cell(long x, long n) {  // check_borders, auxiliary.c:537-544
  x = x % n;
  if (x < 0) x += n;
  return x;
}

// Constants of Rion (user_functions.c:33-38) and pow(1+z, c4), as double bit
// patterns set on the host; qion = Qion(z) for the sfr weight, 0 for Rion.
struct RionConst {
  sd_t c1, c2, c3, three, vnorm, p1, qion;
};

// Rion(hmass, z) = c1 hmass (1+z)^c4 (hmass/c2)^c3 exp(-(c2/hmass)^3) / V_norm
// in double; the value CIC receives is that double (or sfr = Rion / Qion,
// user_functions.c:71-75) rounded to its float parameter (auxiliary.c:761).
__device__ __forceinline__ float weight_sd(float m, const RionConst& k) {
  const sd_t M = sd_from_float(m);
  const sd_t t1 = sd_mul(sd_mul(k.c1, M), k.p1);
  const sd_t t2 = sd_pow(sd_div(M, k.c2), k.c3);
  const sd_t t3 = sd_exp(sd_neg(sd_pow(sd_div(k.c2, M), k.three)));
  const sd_t rion = sd_div(sd_mul(sd_mul(t1, t2), t3), k.vnorm);
  return sd_to_float(k.qion ? sd_div(rion, k.qion) : rion);
}

// 8 contributions per halo, in the reference's corner order.
__global__ void k_halo_contrib(long nh, const HaloRec* __restrict__ halos, RionConst rk, long N,
                               unsigned long long* __restrict__ keys, uint32_t* __restrict__ seq,
                               sd_t* __restrict__ vals) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += (long)gridDim.x * blockDim.x) {
    const HaloRec h = halos[i];
    const float map_in = weight_sd(h.Mass, rk);
    float x1 = h.x, y1 = h.y, z1 = h.z;
    long x = (long)x1, y = (long)y1, z = (long)z1;
    x1 -= (float)x;
    y1 -= (float)y;
    z1 -= (float)z;
    int corner = 0;
    for (long a = 0; a < 2; a++)
      for (long b = 0; b < 2; b++)
        for (long c = 0; c < 2; c++) {
          x += a;
          y += b;
          z += c;
          if (x1 < 0.0f) { x = x - 1; x1 = fabsf(x1); }
          if (y1 < 0.0f) { y = y - 1; y1 = fabsf(y1); }
          if (z1 < 0.0f) { z = z - 1; z1 = fabsf(z1); }
          x = wrap_cell(x, N);
          y = wrap_cell(y, N);
          z = wrap_cell(z, N);
          if (a == 1) x1 = 1.0f - x1;  // (float)(1.0 - x1): exact difference, one rounding
          if (b == 1) y1 = 1.0f - y1;
          if (c == 1) z1 = 1.0f - z1;
          // (1.0 - x1)*(1.0 - y1)*(1.0 - z1)*map_in in double (the differences are exact)
          const sd_t one = 0x3FF0000000000000ULL;
          const sd_t w = sd_mul(sd_mul(sd_mul(sd_sub(one, sd_from_float(x1)), sd_sub(one, sd_from_float(y1))),
                                       sd_sub(one, sd_from_float(z1))),
                                sd_from_float(map_in));
          const long e = 8 * i + corner++;
          keys[e] = (unsigned long long)(x * N * N + y * N + z);
          seq[e] = (uint32_t)e;
          vals[e] = w;
          x -= a;
          y -= b;
          z -= c;
          if (a == 1) x1 = 1.0f - x1;
          if (b == 1) y1 = 1.0f - y1;
          if (c == 1) z1 = 1.0f - z1;
        }
  }
}

// Replay each cell's chain map = (float)((double)map + w) in serial order.
__global__ void k_halo_accumulate(long ne, const unsigned long long* __restrict__ keys,
                                  const uint32_t* __restrict__ seq, const sd_t* __restrict__ vals,
                                  float* __restrict__ fine) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += (long)gridDim.x * blockDim.x) {
    if (i > 0 && keys[i - 1] == keys[i]) continue;  // not the first entry of its cell
    float acc = 0.0f;
    long k = i;
    do {
      acc = sd_to_float(sd_add(sd_from_float(acc), vals[seq[k]]));
      ++k;
    } while (k < ne && keys[k] == keys[i]);
    fine[keys[i]] = acc;
  }
}

// Block average (smooth_box): av = sum of the sm^3 fine values in double in
// the reference's loop order, / sm^3, rounded to float; post_div != 0 then
// divides that float by a double and rounds again (get_SFR.c:129-131).
__global__ void k_smooth_box(const float* __restrict__ fine, float* __restrict__ out, long N, long Ns, long sm,
                             sd_t sm3, sd_t post_div) {
  const long n3 = Ns * Ns * Ns;
  for (long o = (long)blockIdx.x * blockDim.x + threadIdx.x; o < n3; o += (long)gridDim.x * blockDim.x) {
    const long i = o / (Ns * Ns), j = (o / Ns) % Ns, p = o % Ns;
    sd_t av = 0;
    for (long a = 0; a < sm; a++)
      for (long b = 0; b < sm; b++)
        for (long c = 0; c < sm; c++)
          av = sd_add(av, sd_from_float(fine[(i * sm + a) * N * N + (j * sm + b) * N + (p * sm + c)]));
    float v = sd_to_float(sd_div(av, sm3));
    if (post_div) v = sd_to_float(sd_div(sd_from_float(v), post_div));
    out[o] = v;
  }
}

static unsigned grid_for(long n) {
  long b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? b : 152 * 32);
}

size_t halo_scratch_bytes(long nh) {
  const long ne = 8 * nh;
  size_t sort_tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (uint32_t*)nullptr, (uint32_t*)nullptr, (int)ne);
  return (size_t)ne * (2 * sizeof(unsigned long long) + 2 * sizeof(uint32_t) + sizeof(sd_t)) + sort_tmp + 4096;
}

static uint64_t bits_of(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
}

static RionConst rion_const(double z, double qion) {
  RionConst rk;
  rk.c1 = bits_of(1.575e39);
  rk.c2 = bits_of(9.367608e+07);
  rk.c3 = bits_of(0.44);
  rk.three = bits_of(3.0);
  rk.vnorm = bits_of(1.e+45);
  rk.p1 = bits_of(pow((1.0 + z), 2.27044695e+00));
  rk.qion = qion != 0.0 ? bits_of(qion) : 0;
  return rk;
}

cudaError_t launch_halo_source(long nh, const void* halos_dev, double z, long N_halo, long N_smooth, float* fine,
                               float* out, void* scratch, size_t scratch_bytes, cudaStream_t st, double qion,
                               double post_div) {
  const RionConst rk = rion_const(z, qion);
  const long ne = 8 * nh;
  const long Nh3 = N_halo * N_halo * N_halo;
  cudaError_t e;
  if ((e = cudaMemsetAsync(fine, 0, sizeof(float) * Nh3, st))) return e;
  if (nh > 0) {
    unsigned char* p = (unsigned char*)scratch;
    unsigned long long* k0 = (unsigned long long*)p;
    p += ne * sizeof(unsigned long long);
    unsigned long long* k1 = (unsigned long long*)p;
    p += ne * sizeof(unsigned long long);
    uint32_t* s0 = (uint32_t*)p;
    p += ne * sizeof(uint32_t);
    uint32_t* s1 = (uint32_t*)p;
    p += ne * sizeof(uint32_t);
    sd_t* vals = (sd_t*)p;
    p += ne * sizeof(sd_t);
    p = (unsigned char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    size_t tmp_bytes = scratch_bytes - (size_t)(p - (unsigned char*)scratch);
    k_halo_contrib<<<grid_for(nh), 256, 0, st>>>(nh, (const HaloRec*)halos_dev, rk, N_halo, k0, s0, vals);
    if ((e = cudaGetLastError())) return e;
    int end_bit = 1;
    while (end_bit < 64 && ((unsigned long long)1 << end_bit) < (unsigned long long)Nh3) ++end_bit;
    if ((e = cub::DeviceRadixSort::SortPairs(p, tmp_bytes, k0, k1, s0, s1, (int)ne, 0, end_bit, st))) return e;
    k_halo_accumulate<<<grid_for(ne), 256, 0, st>>>(ne, k1, s1, vals, fine);
    if ((e = cudaGetLastError())) return e;
  }
  long sm = (long)roundf((float)((1.0 * N_halo) / N_smooth));
  if (N_smooth * sm > N_halo) sm = sm - 1;
  const double sm3d = 1.0 * sm * sm * sm;
  uint64_t sm3;
  memcpy(&sm3, &sm3d, 8);
  k_smooth_box<<<grid_for(N_smooth * N_smooth * N_smooth), 256, 0, st>>>(
      fine, out, N_halo, N_smooth, sm, sm3, post_div != 0.0 ? bits_of(post_div) : 0);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free variant (sf21_hii_halo_source_noalloc).  Some callers cannot
// call cudaMalloc at the point where they need the source box: a host
// application that owns a fixed device-memory budget and forbids allocations
// after start-up, a caller running between CUDA graph launches that must not
// change the device heap, or one that calls from inside a memory pool's
// callbacks.  For them the fine grid, the sort keys/values and CUB's temporary
// storage live in this fixed file-scope array instead of cudaMalloc'd scratch,
// which caps the sizes (kNoAllocMaxNHalo, kNoAllocMaxHalos).  One array per
// device: calls that overlap on the same device (two streams, two threads)
// share it and race; the caller serialises them.
constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB
constexpr long kNoAllocMaxNHalo = 128;                     // fine grid <= 8 MiB
constexpr long kNoAllocMaxHalos = 16384;                   // 131072 CIC entries, 4 MiB
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kNoAllocMaxDevices];

// Set-up, once per device with that device current: the device address of
// the array.  Nothing is allocated (the array belongs to the loaded module).
static cudaError_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int halo_source_noalloc(double z, long N_halo, long N_smooth, long nh, const void* halos_dev, float* out,
                        cudaStream_t st, char* err, size_t errlen) {
  if (nh < 0 || (nh > 0 && !halos_dev) || !out || N_smooth < 1 || N_halo < 1) {
    snprintf(err, errlen, "bad arguments");
    return SF21_E_ARG;
  }
  if (N_halo < N_smooth) {
    snprintf(err, errlen, "N_halo < N_smoothed (smooth_box, auxiliary.c:651-654)");
    return SF21_E_ARG;
  }
  if (N_halo > kNoAllocMaxNHalo || nh > kNoAllocMaxHalos) {
    snprintf(err, errlen, "no-alloc halo source limited to N_halo <= %ld and <= %ld halos (got N_halo %ld, %ld halos)",
             kNoAllocMaxNHalo, kNoAllocMaxHalos, N_halo, nh);
    return SF21_E_UNSUPPORTED;
  }
  const long ne = 8 * nh;
  const long Nh3 = N_halo * N_halo * N_halo;
  size_t sort_tmp = 0;
  if (ne > 0)
    cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (uint32_t*)nullptr, (uint32_t*)nullptr, (int)ne);
  // layout: fine | k0 | k1 | s0 | s1 | vals | CUB temp, each 256-byte aligned
  const size_t o_k0 = align256(sizeof(float) * Nh3);
  const size_t o_k1 = o_k0 + align256(ne * sizeof(unsigned long long));
  const size_t o_s0 = o_k1 + align256(ne * sizeof(unsigned long long));
  const size_t o_s1 = o_s0 + align256(ne * sizeof(uint32_t));
  const size_t o_v = o_s1 + align256(ne * sizeof(uint32_t));
  const size_t o_t = o_v + align256(ne * sizeof(sd_t));
  if (o_t + sort_tmp > kNoAllocScratchBytes) {
    snprintf(err, errlen, "no-alloc halo source needs %zu scratch bytes, has %zu", o_t + sort_tmp,
             kNoAllocScratchBytes);
    return SF21_E_UNSUPPORTED;
  }
  void* base = nullptr;
  cudaError_t e = noalloc_scratch(&base);
  if (e != cudaSuccess) {
    snprintf(err, errlen, "scratch set-up failed: %s", cudaGetErrorString(e));
    return SF21_E_CUDA;
  }
  unsigned char* p = (unsigned char*)base;
  float* fine = (float*)p;
  const RionConst rk = rion_const(z, 0.0);
  // The fine grid is the only part that must start at zero (the CIC chains
  // write each touched cell once, untouched cells stay 0); keys, sequence
  // numbers and values are written in full before they are read, and CUB
  // initialises its own temporary storage.
  if ((e = cudaMemsetAsync(fine, 0, sizeof(float) * Nh3, st)) == cudaSuccess && nh > 0) {
    unsigned long long* k0 = (unsigned long long*)(p + o_k0);
    unsigned long long* k1 = (unsigned long long*)(p + o_k1);
    uint32_t* s0 = (uint32_t*)(p + o_s0);
    uint32_t* s1 = (uint32_t*)(p + o_s1);
    sd_t* vals = (sd_t*)(p + o_v);
    k_halo_contrib<<<grid_for(nh), 256, 0, st>>>(nh, (const HaloRec*)halos_dev, rk, N_halo, k0, s0, vals);
    e = cudaGetLastError();
    int end_bit = 1;
    while (end_bit < 64 && ((unsigned long long)1 << end_bit) < (unsigned long long)Nh3) ++end_bit;
    if (e == cudaSuccess) e = cub::DeviceRadixSort::SortPairs(p + o_t, sort_tmp, k0, k1, s0, s1, (int)ne, 0, end_bit, st);
    if (e == cudaSuccess) {
      k_halo_accumulate<<<grid_for(ne), 256, 0, st>>>(ne, k1, s1, vals, fine);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) {
    long sm = (long)roundf((float)((1.0 * N_halo) / N_smooth));
    if (N_smooth * sm > N_halo) sm = sm - 1;
    k_smooth_box<<<grid_for(N_smooth * N_smooth * N_smooth), 256, 0, st>>>(fine, out, N_halo, N_smooth, sm,
                                                                           bits_of(1.0 * sm * sm * sm), 0);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    snprintf(err, errlen, "no-alloc halo source: %s", cudaGetErrorString(e));
    return SF21_E_CUDA;
  }
  return SF21_OK;
}

}  // namespace sf21

// Context-free, allocation-free halo source box (declared in sf21_hii.h).
extern "C" int sf21_hii_halo_source_noalloc(double z, long N_halo, long N_smoothed, long nhalos,
                                            const void* halos_dev, float* rion_box_dev, void* stream) {
  char err[256] = {0};
  const int rc = sf21::halo_source_noalloc(z, N_halo, N_smoothed, nhalos, halos_dev, rion_box_dev,
                                           (cudaStream_t)stream, err, sizeof err);
  if (rc != SF21_OK) sf21::set_global_error(err);
  return rc;
}
