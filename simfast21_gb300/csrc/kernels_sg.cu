// Subgrid Poisson cycle of the halo finder on the GPU (get_halos.c:326-371).
//
// The reference walks the unflagged cells in index order and draws one
// Poisson deviate per cell from a single taus generator (gsl_ran_poisson,
// the product-of-uniforms method for means <= 10): a draw that starts at
// stream position s consumes L(s) uniforms, L(s) = the first L with
// u_s u_{s+1} ... u_{s+L-1} <= exp(-mu) (products in double), and returns
// k = L(s) - 1.  Draw n starts at s_n, s_{n+1} = s_n + L(s_n).  The GPU form
// reproduces that stream exactly:
//   A  per block of SG_B positions: the generator's state is jumped to the
//      block (the generator is linear over GF(2): 32x32 bit matrices of its
//      powers), each thread steps 4 consecutive positions, L(s) is computed
//      for every position (one integer compare decides L = 1; longer chains
//      multiply with the IEEE double rounding done in integers), and pointer
//      jumping gives, for every entry
//      offset e < SG_LMAX, the block's exit offset and draw count;
//   B  the entries of all blocks follow by composing those tables (groups of
//      SG_G blocks, supergroups of SG_G groups, in parallel; the supergroups
//      in order; then down to the groups and the blocks);
//   C  each block replays its chain from its entry and lists the draws with
//      k >= 1 (k = 0 writes nothing) with their draw index;
//   D  draw n belongs to the n-th unflagged cell (binary search in the
//      per-word prefix counts of the unflagged bit set); nn = (int)
//      round(k (1 + delta growth hbias)) in soft-double; the records follow
//      from a prefix sum over nn.
// No FP64 unit is used: sg_dmul.h (the draw products) and softdouble.h (the
// halo counts) give the IEEE results in integer arithmetic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf21_kernels.h"
#include "sg_dmul.h"
#include "softdouble.h"

namespace sf21 {

__device__ __forceinline__ uint32_t gf2_apply(const uint32_t* __restrict__ col, uint32_t v) {
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < 32; ++k) r ^= (0u - ((v >> k) & 1u)) & __ldg(col + k);
  return r;
}

// the same with the columns SG_LOCAL words apart
__device__ __forceinline__ uint32_t gf2_apply_strided(const uint32_t* __restrict__ col, uint32_t v) {
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < 32; ++k) r ^= (0u - ((v >> k) & 1u)) & __ldg(col + (size_t)k * SG_LOCAL);
  return r;
}

__device__ __forceinline__ void taus_step(uint32_t& a, uint32_t& b, uint32_t& c) {
  a = ((a & 4294967294u) << 12) ^ (((a << 13) ^ a) >> 19);
  b = ((b & 4294967288u) << 4) ^ (((b << 2) ^ b) >> 25);
  c = ((c & 4294967280u) << 17) ^ (((c << 3) ^ c) >> 11);
}

// Access checks of the draw and record kernels: an index outside its buffer
// is recorded (err[1] = site, err[2] = low 31 bits of the index) and the
// access skipped; the host turns a record into an error return.
__device__ __forceinline__ void sg_bad(int* err, int site, uint64_t idx) {
  if (atomicCAS(err + 1, 0, site) == 0) err[2] = (int)(idx & 0x7fffffff);
}

// A ------------------------------------------------------------------------
// jumps: pow2[(k 3 + c) 32 + col] = column col of component c of T^(2^k)
// (k < SG_POW2); local[(c 32 + col) SG_LOCAL + i] = the same of T^(4 i)
// (i < SG_LOCAL), stored so that the threads of a warp, each applying its own
// power, read consecutive words.  S0: the state whose next step gives
// position 0.
// The state at the start of every block, T^(b SG_B) S0: one thread per
// (block, component), so the jumps of all blocks run in parallel instead of
// keeping a block's other threads waiting.
__global__ void k_sg_start(SgArgs a, const uint32_t* __restrict__ pow2, long nblocks, uint32_t* __restrict__ start) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nblocks * 3) return;
  const long b = t / 3;
  const int c = (int)(t % 3);
  const uint64_t base = (uint64_t)b * SG_B;
  uint32_t v = a.s0[c];
  for (int k = 0; k < SG_POW2; ++k)
    if ((base >> k) & 1u) v = gf2_apply(pow2 + ((size_t)k * 3 + c) * 32, v);
  start[t] = v;
}

__global__ void __launch_bounds__(SG_THREADS)
k_sg_len(SgArgs a, const uint32_t* __restrict__ start, const uint32_t* __restrict__ local, uint8_t* __restrict__ Lout,
         uint32_t* __restrict__ LB, uint8_t* __restrict__ X, uint16_t* __restrict__ D, int* __restrict__ err) {
  __shared__ uint32_t sx[SG_B + SG_LMAX];
  __shared__ uint16_t nxt[SG_B], cnt[SG_B];
  const long b = blockIdx.x;
  const uint64_t base = (uint64_t)b * SG_B;
  const uint32_t sS[3] = {__ldg(start + 3 * b), __ldg(start + 3 * b + 1), __ldg(start + 3 * b + 2)};
  for (int pass = 0; pass < 2; ++pass) {
    const int i0 = pass ? SG_B + 4 * threadIdx.x : 4 * threadIdx.x;
    if (pass && 4 * (int)threadIdx.x >= SG_LMAX) break;
    const uint32_t* J = local + i0 / 4;
    uint32_t x = gf2_apply_strided(J, sS[0]), y = gf2_apply_strided(J + 32 * SG_LOCAL, sS[1]),
             z = gf2_apply_strided(J + 64 * SG_LOCAL, sS[2]);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      taus_step(x, y, z);
      sx[i0 + r] = x ^ y ^ z;
    }
  }
  __syncthreads();
  // L(s): x <= X1 <=> u = x 2^-32 <= exp(-mu) <=> one uniform
  const DMant emu = dm_from_bits(a.emu);
  uint32_t packed = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = 4 * threadIdx.x + r;
    int L = 1;
    const uint32_t xv = sx[i];
    if (xv > a.x1) {  // u_0 > exp(-mu) > 0, so xv > 0
      DMant prod = dm_from_u32(xv);
      for (L = 2; L <= SG_LMAX; ++L) {
        const uint32_t xn = sx[i + L - 1];
        if (xn == 0) break;  // a zero factor ends the draw
        prod = dm_mul_u32(prod, xn);
        if (dm_le(prod, emu)) break;
      }
      if (L > SG_LMAX) {
        atomicOr(err, 1);
        L = SG_LMAX;
      }
    }
    packed |= (uint32_t)L << (8 * r);
    nxt[i] = (uint16_t)(i + L);
    cnt[i] = 1;
  }
  reinterpret_cast<uint32_t*>(Lout + base)[threadIdx.x] = packed;
  // bit set of the positions whose draw takes two uniforms or more (k >= 1):
  // 4 bits per thread, 8 threads per word
  uint32_t nib = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) nib |= (((packed >> (8 * r)) & 0xFFu) >= 2u ? 1u : 0u) << r;
  uint32_t word = nib << (4 * (threadIdx.x & 7));
  word |= __shfl_xor_sync(0xffffffffu, word, 1);
  word |= __shfl_xor_sync(0xffffffffu, word, 2);
  word |= __shfl_xor_sync(0xffffffffu, word, 4);
  if ((threadIdx.x & 7) == 0) LB[(size_t)b * (SG_B / 32) + (threadIdx.x >> 3)] = word;
  __syncthreads();
  // pointer jumping: after log2(SG_B) rounds every chain has left the block
  for (int round = 0; (1 << round) < SG_B; ++round) {
    uint16_t nn[4], cc[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = 4 * threadIdx.x + r;
      const int n = nxt[i];
      if (n < SG_B) {
        nn[r] = nxt[n];
        cc[r] = (uint16_t)(cnt[i] + cnt[n]);
      } else {
        nn[r] = (uint16_t)n;
        cc[r] = cnt[i];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      nxt[4 * threadIdx.x + r] = nn[r];
      cnt[4 * threadIdx.x + r] = cc[r];
    }
    __syncthreads();
  }
  if (threadIdx.x < SG_LMAX) {
    X[(size_t)b * SG_LMAX + threadIdx.x] = (uint8_t)(nxt[threadIdx.x] - SG_B);
    D[(size_t)b * SG_LMAX + threadIdx.x] = cnt[threadIdx.x];
  }
}

// B ------------------------------------------------------------------------
// Entries of all blocks, by composing the per-block tables (exit offset X,
// draws D for each entry offset e < SG_LMAX) in groups of SG_G: blocks ->
// groups -> supergroups (SG_LMAX threads per parent, each walking one entry
// through the SG_G children), one thread over the supergroups, then down again
// (one thread per parent walking its children from the parent's entry).
template <class TD>
__global__ void k_sg_compose(const uint8_t* __restrict__ X, const TD* __restrict__ D, long n,
                             uint8_t* __restrict__ PX, uint32_t* __restrict__ PD) {
  const long g = blockIdx.x;
  const int e0 = threadIdx.x;  // SG_LMAX threads
  int e = e0;
  uint32_t tot = 0;
  const long c1 = (g + 1) * SG_G < n ? (g + 1) * SG_G : n;
  for (long c = g * SG_G; c < c1; ++c) {
    tot += D[(size_t)c * SG_LMAX + e];
    e = X[(size_t)c * SG_LMAX + e];
  }
  PX[(size_t)g * SG_LMAX + e0] = (uint8_t)e;
  PD[(size_t)g * SG_LMAX + e0] = tot;
}

__global__ void k_sg_top(const uint8_t* __restrict__ X, const uint32_t* __restrict__ D, long n,
                         uint8_t* __restrict__ entry, uint64_t* __restrict__ base_out) {
  if (threadIdx.x || blockIdx.x) return;
  int e = 0;
  uint64_t base = 0;
  for (long c = 0; c < n; ++c) {
    entry[c] = (uint8_t)e;
    base_out[c] = base;
    base += D[(size_t)c * SG_LMAX + e];
    e = X[(size_t)c * SG_LMAX + e];
  }
  base_out[n] = base;  // draws available in all generated positions
}

template <class TD>
__global__ void k_sg_descend(const uint8_t* __restrict__ X, const TD* __restrict__ D, long n, long nparents,
                             const uint8_t* __restrict__ pentry, const uint64_t* __restrict__ pbase,
                             uint8_t* __restrict__ entry, uint64_t* __restrict__ base_out) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nparents) return;
  int e = pentry[g];
  uint64_t base = pbase[g];
  const long c1 = (g + 1) * SG_G < n ? (g + 1) * SG_G : n;
  for (long c = g * SG_G; c < c1; ++c) {
    entry[c] = (uint8_t)e;
    base_out[c] = base;
    base += D[(size_t)c * SG_LMAX + e];
    e = X[(size_t)c * SG_LMAX + e];
  }
}

// C ------------------------------------------------------------------------
// mode 0: count the draws with k >= 1 among draws < U per block, and record
// the position after draw U - 1; mode 1: write them (draw index, k).
constexpr int WALK_THREADS = 128;
// Each thread walks one block.  Between two long draws (k >= 1) every draw
// takes one uniform, so the walk jumps from long position to long position
// with the block's bit set of long positions (LB) and counts the one-uniform
// draws in between; it touches the draw lengths (L) only at long positions.
__global__ void __launch_bounds__(WALK_THREADS)
k_sg_walk(int mode, const uint8_t* __restrict__ Lb, const uint32_t* __restrict__ LB, long nblocks,
          const uint8_t* __restrict__ bentry, const uint64_t* __restrict__ bbase, uint64_t U,
          uint32_t* __restrict__ cnt, uint64_t* __restrict__ consumed, uint64_t* __restrict__ dn,
          uint8_t* __restrict__ dk, uint64_t cap, int* __restrict__ err) {
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  uint64_t n = bbase[b];
  if (n >= U) {
    if (mode == 0) cnt[b] = 0;
    return;
  }
  const uint64_t base = (uint64_t)b * SG_B;
  const uint32_t* lb = LB + (size_t)b * (SG_B / 32);
  int s = bentry[b];
  uint32_t c = 0;
  const uint32_t off = mode ? cnt[b] : 0;
  while (s < SG_B && n < U) {
    // next long position p >= s (SG_B if none)
    int w = s >> 5;
    uint32_t m = __ldg(lb + w) & (0xffffffffu << (s & 31));
    while (!m && ++w < SG_B / 32) m = __ldg(lb + w);
    const int p = m ? w * 32 + __ffs(m) - 1 : SG_B;
    // draws at s .. p-1 take one uniform each
    const uint64_t steps = (uint64_t)(p - s);
    if (n + steps >= U) {  // draw U - 1 is one of them
      if (mode == 0) *consumed = base + s + (U - 1 - n) + 1;
      n = U;
      break;
    }
    n += steps;
    s = p;
    if (s >= SG_B) break;
    const int L = Lb[base + s];
    if (mode) {
      if ((uint64_t)off + c < cap) {
        dn[off + c] = n;
        dk[off + c] = (uint8_t)(L - 1);
      } else {
        sg_bad(err, 1, (uint64_t)off + c);
      }
    }
    ++c;
    if (mode == 0 && n == U - 1) *consumed = base + s + L;
    s += L;
    ++n;
  }
  if (mode == 0) cnt[b] = c;
}

// D ------------------------------------------------------------------------
__device__ __forceinline__ int64_t sd_round_half_away(sd_t x) {
  if (sd_is_zero(x)) return 0;
  const int e = (int)((x >> 52) & 0x7FF) - 1023;
  const uint64_t m = (x & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);  // value = m 2^(e-52)
  int64_t q;
  if (e < -1) {
    q = 0;
  } else if (e >= 52) {
    q = (int64_t)(m << (e - 52 < 11 ? e - 52 : 10));
  } else {
    const int sh = 52 - e;  // 1..53
    const uint64_t r = m & ((1ULL << sh) - 1);
    q = (int64_t)(m >> sh) + (r >= (1ULL << (sh - 1)) ? 1 : 0);
  }
  return (x >> 63) ? -q : q;
}

// cell of draw n: the n-th zero bit of FL; wpre[w] = zero bits of words < w
__device__ __forceinline__ uint32_t select_unflagged(const uint32_t* __restrict__ FL,
                                                     const uint32_t* __restrict__ wpre, long nwords, uint64_t n) {
  long lo = 0, hi = nwords - 1;  // last w with wpre[w] <= n
  while (lo < hi) {
    const long mid = (lo + hi + 1) >> 1;
    if (wpre[mid] <= n) lo = mid; else hi = mid - 1;
  }
  uint32_t free_bits = ~FL[lo];
  uint32_t r = (uint32_t)(n - wpre[lo]);
  while (r-- && free_bits) free_bits &= free_bits - 1;
  return (uint32_t)(lo * 32 + (free_bits ? __ffs(free_bits) - 1 : 0));  // n < free cells: never the 0 case
}

__global__ void k_sg_nn(const uint64_t* __restrict__ dn, const uint8_t* __restrict__ dk, long nd,
                        const uint32_t* __restrict__ FL, const uint32_t* __restrict__ wpre, long nwords,
                        const float* __restrict__ delta, uint64_t growth, uint64_t hbias, uint32_t* __restrict__ cell,
                        uint32_t* __restrict__ nn, int* __restrict__ err) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (long)gridDim.x * blockDim.x) {
    const uint32_t t = select_unflagged(FL, wpre, nwords, dn[i]);
    if ((long)t >= nwords * 32) {
      sg_bad(err, 2, t);
      cell[i] = 0;
      nn[i] = 0;
      continue;
    }
    // tempv = map_in_f[index] * growth * hbias; nn = (int) round(Pn (1 + tempv))  (:351-354)
    const sd_t tempv = sd_mul(sd_mul(sd_from_float(delta[t]), growth), hbias);
    const sd_t v = sd_mul(sd_from_int(dk[i]), sd_add(0x3FF0000000000000ULL, tempv));
    int64_t q = sd_round_half_away(v);
    if (q > (1 << 24)) {  // a finite density and k <= 63 stay far below
      sg_bad(err, 3, (uint64_t)i);
      q = 0;
    }
    cell[i] = t;
    nn[i] = q > 0 ? (uint32_t)q : 0u;
  }
}

__global__ void k_sg_records(const uint32_t* __restrict__ cell, const uint32_t* __restrict__ nn,
                             const uint32_t* __restrict__ off, long nd, int N, float mass,
                             float4* __restrict__ out, uint64_t cap, int* __restrict__ err) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (long)gridDim.x * blockDim.x) {
    const uint32_t t = cell[i];
    const uint32_t q = t / (uint32_t)N, a = q / (uint32_t)N;
    const float4 rec = make_float4(mass, (float)a, (float)(q - a * (uint32_t)N), (float)(t - q * (uint32_t)N));
    const uint32_t o = off[i];
    for (uint32_t r = 0; r < nn[i]; ++r) {
      if ((uint64_t)o + r < cap)
        out[o + r] = rec;
      else
        sg_bad(err, 4, (uint64_t)o + r);
    }
  }
}

// zero bits per word of FL
__global__ void k_sg_free_count(const uint32_t* __restrict__ FL, long nwords, uint32_t* __restrict__ c) {
  for (long w = (long)blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += (long)gridDim.x * blockDim.x)
    c[w] = 32u - (uint32_t)__popc(FL[w]);
}

// ---------------------------------------------------------------------------
// Exclusive prefix sums of a uint32 array (chunk sums, one CTA over the
// chunk sums, per-chunk scans with the chunk's offset).  Totals < 2^32.
constexpr int SC_THREADS = 256;
constexpr long SC_CHUNK = 8192;

__global__ void __launch_bounds__(SC_THREADS) k_chunk_sum(const uint32_t* __restrict__ a, long n,
                                                          uint32_t* __restrict__ sums) {
  const long c0 = blockIdx.x * SC_CHUNK;
  uint32_t s = 0;
  for (long i = c0 + threadIdx.x; i < c0 + SC_CHUNK && i < n; i += SC_THREADS) s += a[i];
  s = __reduce_add_sync(0xffffffffu, s);
  __shared__ uint32_t red[SC_THREADS / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int k = 0; k < SC_THREADS / 32; ++k) t += red[k];
    sums[blockIdx.x] = t;
  }
}

// a and out may be the same array (in-place scans): no __restrict__ on
// them, so every element is loaded before its slot is overwritten.
__global__ void __launch_bounds__(SC_THREADS) k_chunk_scan(const uint32_t* a, long n,
                                                           const uint32_t* __restrict__ off, uint32_t* out) {
  // each thread scans SC_CHUNK / SC_THREADS consecutive elements
  constexpr int PER = (int)(SC_CHUNK / SC_THREADS);
  const long i0 = blockIdx.x * SC_CHUNK + (long)threadIdx.x * PER;
  uint32_t s = 0;
  for (int k = 0; k < PER; ++k)
    if (i0 + k < n) s += a[i0 + k];
  __shared__ uint32_t wsum[SC_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int k = 0; k < w; ++k) before += wsum[k];
  uint32_t run = off[blockIdx.x] + before + x - s;
  for (int k = 0; k < PER; ++k) {
    if (i0 + k >= n) break;
    const uint32_t v = a[i0 + k];
    out[i0 + k] = run;
    run += v;
  }
}

long scan_chunks(long n) { return (n + SC_CHUNK - 1) / SC_CHUNK; }

cudaError_t launch_scan_u32(const uint32_t* a, long n, uint32_t* out, uint32_t* chunk, uint32_t* total,
                            cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long nc = scan_chunks(n);
  k_chunk_sum<<<(unsigned)nc, SC_THREADS, 0, st>>>(a, n, chunk);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  if ((e = launch_scan_counts(chunk, nc, total, st))) return e;
  k_chunk_scan<<<(unsigned)nc, SC_THREADS, 0, st>>>(a, n, chunk, out);
  return cudaGetLastError();
}

static unsigned grid_for(long n, int threads) {
  long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)b;
}

cudaError_t launch_sg_len(long nblocks, const SgArgs& a, const uint32_t* pow2, const uint32_t* local, uint32_t* start,
                          uint8_t* L, uint32_t* LB, uint8_t* X, uint16_t* D, int* err, cudaStream_t st) {
  k_sg_start<<<(unsigned)((nblocks * 3 + 255) / 256), 256, 0, st>>>(a, pow2, nblocks, start);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  k_sg_len<<<(unsigned)nblocks, SG_THREADS, 0, st>>>(a, start, local, L, LB, X, D, err);
  return cudaGetLastError();
}

long sg_groups(long n) { return (n + SG_G - 1) / SG_G; }

cudaError_t launch_sg_entries(const uint8_t* X, const uint16_t* D, long nblocks, const SgEntryBufs& eb,
                              cudaStream_t st) {
  const long ng = sg_groups(nblocks), ns = sg_groups(ng);
  k_sg_compose<uint16_t><<<(unsigned)ng, SG_LMAX, 0, st>>>(X, D, nblocks, eb.gx, eb.gd);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  k_sg_compose<uint32_t><<<(unsigned)ns, SG_LMAX, 0, st>>>(eb.gx, eb.gd, ng, eb.sx, eb.sd);
  if ((e = cudaGetLastError())) return e;
  k_sg_top<<<1, 32, 0, st>>>(eb.sx, eb.sd, ns, eb.sentry, eb.sbase);
  if ((e = cudaGetLastError())) return e;
  k_sg_descend<uint32_t><<<(unsigned)((ns + 127) / 128), 128, 0, st>>>(eb.gx, eb.gd, ng, ns, eb.sentry, eb.sbase,
                                                                        eb.gentry, eb.gbase);
  if ((e = cudaGetLastError())) return e;
  k_sg_descend<uint16_t><<<(unsigned)((ng + 127) / 128), 128, 0, st>>>(X, D, nblocks, ng, eb.gentry, eb.gbase,
                                                                        eb.bentry, eb.bbase);
  return cudaGetLastError();
}

cudaError_t launch_sg_walk(int mode, const uint8_t* L, const uint32_t* LB, long nblocks, const uint8_t* bentry,
                           const uint64_t* bbase, uint64_t U, uint32_t* cnt, uint64_t* consumed, uint64_t* dn,
                           uint8_t* dk, uint64_t cap, int* err, cudaStream_t st) {
  k_sg_walk<<<(unsigned)((nblocks + WALK_THREADS - 1) / WALK_THREADS), WALK_THREADS, 0, st>>>(
      mode, L, LB, nblocks, bentry, bbase, U, cnt, consumed, dn, dk, cap, err);
  return cudaGetLastError();
}

cudaError_t launch_sg_free_count(const uint32_t* FL, long nwords, uint32_t* c, cudaStream_t st) {
  k_sg_free_count<<<grid_for(nwords, 256), 256, 0, st>>>(FL, nwords, c);
  return cudaGetLastError();
}

cudaError_t launch_sg_nn(const uint64_t* dn, const uint8_t* dk, long nd, const uint32_t* FL, const uint32_t* wpre,
                         long nwords, const float* delta, uint64_t growth, uint64_t hbias, uint32_t* cell,
                         uint32_t* nn, int* err, cudaStream_t st) {
  if (nd <= 0) return cudaSuccess;
  k_sg_nn<<<grid_for(nd, 256), 256, 0, st>>>(dn, dk, nd, FL, wpre, nwords, delta, growth, hbias, cell, nn, err);
  return cudaGetLastError();
}

cudaError_t launch_sg_records(const uint32_t* cell, const uint32_t* nn, const uint32_t* off, long nd, int N,
                              float mass, float4* out, uint64_t cap, int* err, cudaStream_t st) {
  if (nd <= 0) return cudaSuccess;
  k_sg_records<<<grid_for(nd, 256), 256, 0, st>>>(cell, nn, off, nd, N, mass, out, cap, err);
  return cudaGetLastError();
}

}  // namespace sf21
