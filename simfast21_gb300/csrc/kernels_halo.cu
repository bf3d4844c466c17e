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
// ones) and written at its serial position, the (cell, weight) entries are
// grouped by cell with a stable radix sort (the serial order survives inside
// each cell), and each cell's chain is replayed in that order.  The block
// average gives the reference's serial double sum (exactly, by an integer sum
// when no partial sum rounds, else by the soft-double chain).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>
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
  if (x >= 0 && x < n) return x;  // the usual cases without a 64-bit division
  if (x >= n && x < 2 * n) return x - n;
  if (x < 0 && x >= -n) return x + n;
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

// Weights per distinct mass.  A catalogue of the halo finder holds a few
// distinct masses (one per mass of its schedule), so the soft-double
// pow/exp of the weight runs once per distinct mass: the mass bit patterns
// are sorted and made unique, their weights computed, and each halo finds
// its mass by binary search.
__global__ void k_mass_keys(long nh, const HaloRec* __restrict__ halos, uint32_t* __restrict__ keys) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += (long)gridDim.x * blockDim.x)
    keys[i] = __float_as_uint(halos[i].Mass);
}

__global__ void k_mass_weights(long nh, const uint32_t* __restrict__ uniq, const int* __restrict__ n_uniq,
                               RionConst rk, float* __restrict__ w) {
  const long n = *n_uniq;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n && i < nh; i += (long)gridDim.x * blockDim.x)
    w[i] = weight_sd(__uint_as_float(uniq[i]), rk);
}

struct MassTable {
  const uint32_t* uniq;  // sorted distinct mass bit patterns (nullptr: compute per halo)
  const int* n_uniq;
  const float* w;
};

// 8 contributions per halo, in the reference's corner order: entry 8 i + c
// holds the cell key and the double weight of corner c of halo i, so the
// entries are in the serial order of the reference's deposit loop.
constexpr int CONTRIB_THREADS = 256;
constexpr int MASS_SMEM = 1024;  // distinct masses held in shared memory

template <typename K>
__global__ void __launch_bounds__(CONTRIB_THREADS)
k_halo_contrib(long nh, const HaloRec* __restrict__ halos, RionConst rk, MassTable mt, long N,
               K* __restrict__ keys, sd_t* __restrict__ vals) {
  __shared__ K skey[8 * CONTRIB_THREADS];
  __shared__ sd_t sval[8 * CONTRIB_THREADS];
  __shared__ uint32_t suniq[MASS_SMEM];
  __shared__ float sw[MASS_SMEM];
  const int nu = mt.uniq ? *mt.n_uniq : 0;
  const bool in_smem = nu > 0 && nu <= MASS_SMEM;
  if (in_smem)
    for (int t = threadIdx.x; t < nu; t += blockDim.x) {
      suniq[t] = mt.uniq[t];
      sw[t] = mt.w[t];
    }
  const uint32_t* uq = in_smem ? suniq : mt.uniq;
  const float* wq = in_smem ? sw : mt.w;
  __syncthreads();
  // one chunk of CONTRIB_THREADS halos per block and step (uniform trip count:
  // the staging barriers are reached by every thread)
  for (long b0 = (long)blockIdx.x * CONTRIB_THREADS; b0 < nh; b0 += (long)gridDim.x * CONTRIB_THREADS) {
    const long i = b0 + threadIdx.x;
    if (i < nh) {
      const HaloRec h = halos[i];
      float map_in;
      if (mt.uniq) {
        // the mass is present: lower bound of its bits in uq[0, nu)
        const uint32_t key = __float_as_uint(h.Mass);
        int lo = 0, hi = nu - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (uq[mid] < key)
            lo = mid + 1;
          else
            hi = mid;
        }
        map_in = wq[lo];
      } else {
        map_in = weight_sd(h.Mass, rk);
      }
      const sd_t mw = sd_from_float(map_in);
      // The reference's corner loop (auxiliary.c:769-806) moves a negative
      // fraction f to the cell below at its first corner, then for each upper
      // corner flips f to (float)(1.0 - f) and back again after the deposit.
      // The flip back is not exact for f < 1/2: it leaves f' = 1 - fl(1 - f),
      // and later corners see f'.  Along each axis the cells are wrap(c0) and
      // wrap(c0 + 1); the factors, in the loop's corner order (a, b, c), are
      //   x: a = 0: 1 - x;  a = 1: 1 - fl(1 - x)
      //   y: b = 0: 1 - y for a = 0, 1 - y' for a = 1;  b = 1: 1 - fl(1 - y)
      //   z: c = 0: 1 - z for (a, b) = (0, 0), 1 - z' after;  c = 1: 1 - fl(1 - z)
      // (1 - v in double, as the reference's (1.0 - x1)), multiplied in the
      // reference's order ((fx * fy) * fz) * map_in.
      const sd_t one = 0x3FF0000000000000ULL;
      float f[3] = {h.x, h.y, h.z};
      long c0[3];
      float fr[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        long c = (long)f[d];
        float q = f[d] - (float)c;
        if (q < 0.0f) {
          c = c - 1;
          q = fabsf(q);
        }
        c0[d] = c;
        fr[d] = q;
      }
      const float fx1 = 1.0f - fr[0], fy1 = 1.0f - fr[1], fz1 = 1.0f - fr[2];  // fl(1 - f)
      const float yp = 1.0f - fy1, zp = 1.0f - fz1;                              // f' (exact differences)
      const sd_t FX[2] = {sd_sub(one, sd_from_float(fr[0])), sd_sub(one, sd_from_float(fx1))};
      const sd_t FY0[2] = {sd_sub(one, sd_from_float(fr[1])), sd_sub(one, sd_from_float(yp))};
      const sd_t FY1 = sd_sub(one, sd_from_float(fy1));
      const sd_t FZ0 = sd_sub(one, sd_from_float(fr[2])), FZ0p = sd_sub(one, sd_from_float(zp));
      const sd_t FZ1 = sd_sub(one, sd_from_float(fz1));
      const long cx[2] = {wrap_cell(c0[0], N), wrap_cell(c0[0] + 1, N)};
      const long cy[2] = {wrap_cell(c0[1], N), wrap_cell(c0[1] + 1, N)};
      const long cz[2] = {wrap_cell(c0[2], N), wrap_cell(c0[2] + 1, N)};
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
          const sd_t xy = sd_mul(FX[a], b ? FY1 : FY0[a]);
          const long kxy = (cx[a] * N + cy[b]) * N;
#pragma unroll
          for (int c = 0; c < 2; c++) {
            const sd_t fz = c ? FZ1 : ((a == 0 && b == 0) ? FZ0 : FZ0p);
            const int slot = 8 * threadIdx.x + 4 * a + 2 * b + c;
            skey[slot] = (K)(kxy + cz[c]);
            sval[slot] = sd_mul(sd_mul(xy, fz), mw);
          }
        }
    }
    __syncthreads();
    // entry 8 i + c of the chunk, written with consecutive threads on
    // consecutive entries
    const long e0 = 8 * b0, ne = 8 * nh;
    for (int t = threadIdx.x; t < 8 * CONTRIB_THREADS; t += CONTRIB_THREADS)
      if (e0 + t < ne) {
        keys[e0 + t] = skey[t];
        vals[e0 + t] = sval[t];
      }
    __syncthreads();
  }
}

// Replay each cell's chain map = (float)((double)map + w) in serial order:
// the entries were sorted by cell with a stable sort, so each cell's run
// keeps the deposit order.
template <typename K>
__global__ void k_halo_accumulate(long ne, const K* __restrict__ keys, const sd_t* __restrict__ vals,
                                  float* __restrict__ fine) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += (long)gridDim.x * blockDim.x) {
    const K key = keys[i];
    if (i > 0 && keys[i - 1] == key) continue;  // not the first entry of its cell
    float acc = 0.0f;
    long k = i;
    do {
      acc = sd_to_float(sd_add(sd_from_float(acc), vals[k]));
      ++k;
    } while (k < ne && keys[k] == key);
    fine[key] = acc;
  }
}

static unsigned grid_for(long n);

static int key_bits(long Nh3) {
  int end_bit = 1;
  while (end_bit < 64 && ((unsigned long long)1 << end_bit) < (unsigned long long)Nh3) ++end_bit;
  return end_bit;
}

// Deposit of nh halos into the zeroed fine grid: contributions, stable sort
// by cell (keys K: 32 bits when N^3 <= 2^32), replay.
template <typename K>
static cudaError_t deposit(long nh, const HaloRec* halos, RionConst rk, MassTable mt, long N, K* k0, K* k1,
                           sd_t* v0, sd_t* v1, void* tmp, size_t tmp_bytes, float* fine, cudaStream_t st) {
  const long ne = 8 * nh;
  k_halo_contrib<K><<<grid_for(nh), CONTRIB_THREADS, 0, st>>>(nh, halos, rk, mt, N, k0, v0);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  if ((e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k0, k1, v0, v1, (int)ne, 0, key_bits(N * N * N), st)))
    return e;
  k_halo_accumulate<K><<<grid_for(ne), 256, 0, st>>>(ne, k1, v1, fine);
  return cudaGetLastError();
}

// Block average (smooth_box): av = sum of the sm^3 fine values in double in
// the reference's loop order, / sm^3, rounded to float; a post divisor then
// divides that float by a double and rounds again (get_SFR.c:129-131).
//
// Fast exact path: when the block's values are non-negative and their
// significands, aligned to the smallest one, sum to less than 2^53, every
// partial sum of the serial double loop is exact, so the loop's result is the
// integer sum; av is then that integer times a power of two.  Otherwise the
// serial soft-double chain runs.  Divisions by sm^3 (when not a power of two)
// and by the post divisor use precomputed reciprocals (sd_div_c).
struct SmoothArgs {
  long N, Ns, sm;
  int sm3_log2;    // log2(sm^3) when a power of two, else -1
  sd_divc sm3;     // sm^3 as a divisor
  int post;        // 1: divide by post_div
  sd_divc post_div;
};

// Exact-path step: adds float bits u to the running sum S * 2^emin;
// returns false when the sum leaves the exact range (or u is negative,
// infinite or NaN).
__device__ __forceinline__ bool exact_add(uint32_t u, uint64_t& S, int& emin) {
  if (u == 0) return true;
  const uint32_t ex = u >> 23;  // sign bit included: negative values leave the fast path
  if (ex >= 0xFF) return false;
  const uint64_t m = ex ? ((u & 0x7FFFFFu) | 0x800000u) : u;
  const int e = ex ? (int)ex - 150 : -149;
  if (S == 0) {
    S = m;
    emin = e;
    return true;
  }
  if (e < emin) {  // rebase the sum on the smaller exponent
    const int d = emin - e;
    if (d > 29 || (S >> (53 - d)) != 0) return false;
    S <<= d;
    emin = e;
  }
  const int sh = e - emin;
  if (sh > 29) return false;
  S += m << sh;
  return (S >> 53) == 0;
}

__device__ __forceinline__ sd_t exact_pack(uint64_t S, int emin) {
  if (S == 0) return 0;
  const int lz = sd_clz64(S);
  const uint64_t m = S << (lz - 11);  // leading one at bit 52
  const int e = emin + (63 - lz);     // S * 2^emin = (m / 2^52) * 2^e
  return ((uint64_t)(e + 1023) << 52) | (m & 0xFFFFFFFFFFFFFULL);
}

// Sum of the n values v[0..n) (loop order) in double, serial semantics.
__device__ __forceinline__ sd_t block_sum(const float* v, int n) {
  uint64_t S = 0;
  int emin = 0;
  bool ok = true;
  for (int k = 0; k < n && ok; k++) ok = exact_add(__float_as_uint(v[k]), S, emin);
  if (ok) return exact_pack(S, emin);
  sd_t av = 0;
  for (int k = 0; k < n; k++) av = sd_add(av, sd_from_float(v[k]));
  return av;
}

__device__ __forceinline__ sd_t smooth_sum(const float* __restrict__ fine, long base, const SmoothArgs& a) {
  const long N = a.N;
  const int sm = (int)a.sm;
  if (sm == 2) {  // the usual case (N_halo = 2 N_smoothed): all eight loads issued together
    float v[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float* row = fine + base + (long)(k >> 1) * N * N + (long)(k & 1) * N;
      v[2 * k] = __ldg(row);
      v[2 * k + 1] = __ldg(row + 1);
    }
    return block_sum(v, 8);
  }
  if (sm == 1) return sd_from_float(fine[base]);
  // other block sides: one row of sm values at a time
  uint64_t S = 0;
  int emin = 0;
  bool ok = true;
  for (int x = 0; x < sm && ok; x++)
    for (int y = 0; y < sm && ok; y++) {
      const float* row = fine + base + (long)x * N * N + (long)y * N;
      for (int z = 0; z < sm && ok; z++) ok = exact_add(__float_as_uint(row[z]), S, emin);
    }
  if (ok) return exact_pack(S, emin);
  sd_t av = 0;
  for (int x = 0; x < sm; x++)
    for (int y = 0; y < sm; y++)
      for (int z = 0; z < sm; z++) av = sd_add(av, sd_from_float(fine[base + (long)x * N * N + (long)y * N + z]));
  return av;
}

// One CTA row per (i, j) of the smoothed box (blockIdx.x = i * Ns + j),
// threads over p.
__global__ void k_smooth_box(const float* __restrict__ fine, float* __restrict__ out, const SmoothArgs a) {
  const long N = a.N, sm = a.sm;
  const int Ns = (int)a.Ns;
  const int p = blockIdx.y * blockDim.x + threadIdx.x;
  if (p >= Ns) return;
  const int i = blockIdx.x / Ns, j = blockIdx.x % Ns;
  const sd_t av = smooth_sum(fine, ((long)i * sm) * N * N + ((long)j * sm) * N + (long)p * sm, a);
  sd_t q;
  if (a.sm3_log2 >= 0)
    // exact: av / 2^k stays normal (a NaN from non-finite input stays NaN)
    q = (sd_is_zero(av) || ((av >> 52) & 0x7FF) == 0x7FF) ? av : av - ((uint64_t)a.sm3_log2 << 52);
  else
    q = sd_div_c(av, a.sm3);
  float v = sd_to_float(q);
  if (a.post) v = sd_to_float(sd_div_c(sd_from_float(v), a.post_div));
  out[(long)blockIdx.x * Ns + p] = v;
}

static SmoothArgs smooth_args(long N_halo, long N_smooth, double post_div) {
  SmoothArgs a;
  long sm = (long)roundf((float)((1.0 * N_halo) / N_smooth));
  if (N_smooth * sm > N_halo) sm = sm - 1;
  a.N = N_halo;
  a.Ns = N_smooth;
  a.sm = sm;
  const double sm3 = 1.0 * sm * sm * sm;
  int k = 0;
  while ((1L << k) < sm * sm * sm) ++k;
  a.sm3_log2 = ((1L << k) == sm * sm * sm) ? k : -1;
  uint64_t b;
  memcpy(&b, &sm3, 8);
  a.sm3 = sd_divc_prepare(b);
  a.post = post_div != 0.0;
  memcpy(&b, &post_div, 8);
  a.post_div = sd_divc_prepare(a.post ? b : 0x3FF0000000000000ULL);
  return a;
}

static cudaError_t launch_smooth(const float* fine, float* out, long N_halo, long N_smooth, double post_div,
                                 cudaStream_t st) {
  const int T = 128;
  const dim3 grid((unsigned)(N_smooth * N_smooth), (unsigned)((N_smooth + T - 1) / T));
  k_smooth_box<<<grid, T, 0, st>>>(fine, out, smooth_args(N_halo, N_smooth, post_div));
  return cudaGetLastError();
}

static unsigned grid_for(long n) {
  long b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? b : 152 * 32);
}

size_t halo_scratch_bytes(long nh) {
  const long ne = 8 * nh;
  size_t t64 = 0, t32 = 0, key_tmp = 0, uniq_tmp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, t64, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (sd_t*)nullptr, (sd_t*)nullptr, (int)ne);
  cub::DeviceRadixSort::SortPairs(nullptr, t32, (uint32_t*)nullptr, (uint32_t*)nullptr, (sd_t*)nullptr,
                                  (sd_t*)nullptr, (int)ne);
  cub::DeviceRadixSort::SortKeys(nullptr, key_tmp, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)nh);
  cub::DeviceSelect::Unique(nullptr, uniq_tmp, (uint32_t*)nullptr, (uint32_t*)nullptr, (int*)nullptr, (int)nh);
  size_t tmp = t64 > t32 ? t64 : t32;
  tmp = tmp > key_tmp ? tmp : key_tmp;
  tmp = tmp > uniq_tmp ? tmp : uniq_tmp;
  // k0 | k1 (8 B each) | v0 | v1 (8 B each) | CUB temporary storage
  return (size_t)ne * 32 + tmp + 4096;
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
    void* k0 = p;
    p += ne * 8;
    void* k1 = p;
    p += ne * 8;
    sd_t* v0 = (sd_t*)p;
    p += ne * sizeof(sd_t);
    sd_t* v1 = (sd_t*)p;
    p += ne * sizeof(sd_t);
    p = (unsigned char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    size_t tmp_bytes = scratch_bytes - (size_t)(p - (unsigned char*)scratch);
    // distinct-mass table (16 nh bytes) and its count in v1, free until the
    // cell sort writes it (64 nh bytes); CUB's temporary storage is the cell
    // sort's
    uint32_t* mk0 = (uint32_t*)v1;
    uint32_t* mk1 = mk0 + nh;
    uint32_t* uniq = mk1 + nh;
    float* wts = (float*)(uniq + nh);
    int* n_uniq = (int*)(wts + nh);
    const HaloRec* hrec = (const HaloRec*)halos_dev;
    k_mass_keys<<<grid_for(nh), 256, 0, st>>>(nh, hrec, mk0);
    if ((e = cudaGetLastError())) return e;
    size_t tb = tmp_bytes;
    if ((e = cub::DeviceRadixSort::SortKeys(p, tb, mk0, mk1, (int)nh, 0, 32, st))) return e;
    tb = tmp_bytes;
    if ((e = cub::DeviceSelect::Unique(p, tb, mk1, uniq, n_uniq, (int)nh, st))) return e;
    k_mass_weights<<<grid_for(nh), 256, 0, st>>>(nh, uniq, n_uniq, rk, wts);
    if ((e = cudaGetLastError())) return e;
    const MassTable mt = {uniq, n_uniq, wts};
    if (key_bits(Nh3) <= 32)
      e = deposit<uint32_t>(nh, hrec, rk, mt, N_halo, (uint32_t*)k0, (uint32_t*)k1, v0, v1, p, tmp_bytes, fine, st);
    else
      e = deposit<unsigned long long>(nh, hrec, rk, mt, N_halo, (unsigned long long*)k0, (unsigned long long*)k1, v0,
                                      v1, p, tmp_bytes, fine, st);
    if (e) return e;
  }
  return launch_smooth(fine, out, N_halo, N_smooth, post_div, st);
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
//
// The array's device address belongs to the CUDA context the module is loaded
// in.  It is looked up with cudaGetSymbolAddress once per context (the first
// call in a context does it, so that call should come before any stream
// capture) and cached under the context's process-unique id (cuCtxGetId):
// after cudaDeviceReset, or under another context, the next call looks it up
// again instead of reusing a stale address.
constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB
constexpr long kNoAllocMaxNHalo = 128;                     // fine grid <= 8 MiB
constexpr long kNoAllocMaxHalos = 16384;                   // 131072 CIC entries, 4 MiB
constexpr int kNoAllocCacheSlots = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static struct {
  unsigned long long ctx_id;
  void* ptr;
} g_noalloc_cache[kNoAllocCacheSlots];
static int g_noalloc_next = 0;

// Process-unique id of the current context (driver entry points, so the
// library needs no link against libcuda).
static cudaError_t current_context_id(unsigned long long* id) {
  typedef int (*CtxGetCurrent)(void**);
  typedef int (*CtxGetId)(void*, unsigned long long*);
  static CtxGetCurrent get_current = nullptr;
  static CtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* f = nullptr;
    void* g = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess)
      return cudaErrorNotSupported;
    get_current = (CtxGetCurrent)f;
    get_id = (CtxGetId)g;
  }
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx) return cudaErrorDeviceUninitialized;
  return get_id(ctx, id) == 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

// Set-up, once per context with its device current: the device address of
// the array.  Nothing is allocated (the array belongs to the loaded module).
static cudaError_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaSetDevice(dev);  // makes the device's primary context current
  unsigned long long id = 0;
  if (e == cudaSuccess) e = current_context_id(&id);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  for (int i = 0; i < kNoAllocCacheSlots; ++i)
    if (g_noalloc_cache[i].ptr && g_noalloc_cache[i].ctx_id == id) {
      *out = g_noalloc_cache[i].ptr;
      return cudaSuccess;
    }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  g_noalloc_cache[g_noalloc_next] = {id, p};
  g_noalloc_next = (g_noalloc_next + 1) % kNoAllocCacheSlots;
  *out = p;
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
  if (ne > 0) {
    const cudaError_t q = cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                                          (sd_t*)nullptr, (sd_t*)nullptr, (int)ne);
    if (q != cudaSuccess) {
      snprintf(err, errlen, "no-alloc halo source: sort size query failed: %s", cudaGetErrorString(q));
      return SF21_E_CUDA;
    }
  }
  // layout: fine | k0 | k1 | v0 | v1 | CUB temp, each 256-byte aligned (N_halo <= 128: 32-bit keys)
  const size_t o_k0 = align256(sizeof(float) * Nh3);
  const size_t o_k1 = o_k0 + align256(ne * sizeof(uint32_t));
  const size_t o_v0 = o_k1 + align256(ne * sizeof(uint32_t));
  const size_t o_v1 = o_v0 + align256(ne * sizeof(sd_t));
  const size_t o_t = o_v1 + align256(ne * sizeof(sd_t));
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
  // write each touched cell once, untouched cells stay 0); keys and values
  // are written in full before they are read, and CUB initialises its own
  // temporary storage.
  if ((e = cudaMemsetAsync(fine, 0, sizeof(float) * Nh3, st)) == cudaSuccess && nh > 0) {
    const MassTable direct = {nullptr, nullptr, nullptr};
    e = deposit<uint32_t>(nh, (const HaloRec*)halos_dev, rk, direct, N_halo, (uint32_t*)(p + o_k0),
                          (uint32_t*)(p + o_k1), (sd_t*)(p + o_v0), (sd_t*)(p + o_v1), p + o_t, sort_tmp, fine, st);
  }
  if (e == cudaSuccess) {
    e = launch_smooth(fine, out, N_halo, N_smooth, 0.0, st);
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
