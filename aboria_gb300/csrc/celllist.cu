// CellListOrdered build (the reference's update_positions for an ordered
// cell list: enforce_domain_lambda, src/NeighbourSearchBase.h:185-238; the
// bucket index of src/detail/SpatialUtil.h:125-138; the stable sort_by_key of
// src/detail/Algorithms.h:173-206; lower_bound/upper_bound per bucket,
// src/CellListOrdered.h:231-239; Particles::reorder, src/Particles.h:694-726)
// as five launches and one device-to-host read:
//
//  1. k_cl_keys      domain enforcement, alive test and bucket key per
//                    particle in one pass over the positions; dead particles
//                    get the key maxkey+1 (so the sort moves them to the end)
//                    instead of a compaction; per-pass digit histograms.
//  2. k_cl_onesweep  one launch per 10-bit digit of a stable LSD radix sort:
//                    tiles claimed in order, per-tile digit counts published
//                    and prefixed by decoupled look-back (no histogram scan
//                    launches).
//  3. k_cl_ranges    bucket_begin/bucket_end of every cell straight from the
//                    sorted keys (each boundary between two keys writes the
//                    cells in its gap; no memset, no scan).
//  4. k_cl_gather    positions, ids and the scalar column into cell order.
//
// The grid depends on the alive count (set_domain_impl,
// src/CellListOrdered.h:132-186).  The build assumes the grid that count n
// (nobody deleted) gives, reads the dead count back at the end, and runs
// again with the right grid in the rare case deletions change it.
//
// Bucket index without the FP64 pipe: v_d = floor(fl(fl(x_d - lo_d) *
// inv_side_d)) is non-decreasing in x_d, so it equals the number of cell
// boundaries b_1..b_size at or below x_d, where b_v is the smallest double
// with index >= v.  The host finds every b_v exactly (its IEEE double
// arithmetic is the device's __dsub_rn/__dmul_rn); the device estimates v in
// FP32 and corrects it by 64-bit integer comparisons of order-preserving bit
// patterns, so keys are bit-identical to the FP64 formula.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "handles.cuh"

namespace abx {
namespace {

constexpr int CL_TPB = 256;
constexpr int CL_ITEMS = 16;
constexpr int CL_TILE = 16384;                         // keys per sort tile
constexpr int SW_TPB = 512;                            // sort-pass threads per block
constexpr int SW_WARPS = SW_TPB / 32;
constexpr int SW_ROUNDS = CL_TILE / (SW_TPB * CL_ITEMS);  // rounds of 16 keys per thread
static_assert(CL_TILE % (SW_TPB * CL_ITEMS) == 0 && (1 << 10) % SW_TPB == 0 && CL_TILE <= 65535,
              "sort tile shape (16-bit counts, whole digits per thread)");
constexpr int CL_BND_SMEM = 4096;  // boundary entries staged in shared memory (32 KB)
constexpr int CL_KEYS_TILE = 4096;                     // particles per keys-kernel step
constexpr int CL_RB = 10;
constexpr int CL_RADIX = 1 << CL_RB;
constexpr int CL_MAX_PASSES = 4;
constexpr uint32_t CL_SPIN_CAP = 1u << 26;   // look-back polls before giving up
constexpr int CL_WRAP_CAP = 1 << 20;         // periodic wrap steps before giving up
constexpr uint64_t ST_AGG = 1ull << 32, ST_INCL = 2ull << 32;

constexpr int CL_HIST_COPIES = 32;  // spread of the keys kernel's histogram atomics

struct ClHeader {
  uint32_t hist[CL_MAX_PASSES][CL_RADIX];
  uint32_t tile_counter[CL_MAX_PASSES];
  uint32_t dead;
  uint32_t error;  // 1: a look-back wait gave up; 2: a periodic wrap did not end
  uint32_t blocks_done;
  // per-block histograms land in one of CL_HIST_COPIES copies (few blocks
  // share a counter), the last block to finish sums them into hist
  uint32_t part[CL_HIST_COPIES][CL_MAX_PASSES][CL_RADIX];
};

struct ClParams {
  int dim, npasses;
  uint32_t size[3];
  double lo[3], hi[3], inv[3];
  int periodic[3];
  uint64_t olo[3], ohi[3];  // order-preserving bit patterns of lo, hi
  float inv_f[3], c_f[3];   // FP32 estimate of the bucket coordinate: x * inv_f + c_f
  float lo_fast[3], hi_fast[3], delta_f[3];  // FP32 fast-path bounds
  const uint64_t *bnd[3];   // size+2 boundaries per dimension (ordered bits)
  const uint64_t *bnd_all;  // all of them, dimension after dimension
  int bnd_off[3], bnd_total;
  uint32_t dead_key;
};

__host__ __device__ __forceinline__ uint64_t ord_bits(uint64_t u) {
  if ((u << 1) == 0) u = 0;  // -0 orders like +0
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

uint64_t ord_host(double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return ord_bits(u);
}

// FP32 value of a double from its bits (truncated mantissa), for the estimate.
__device__ __forceinline__ float approx_f32(uint64_t u) {
  const uint32_t hi = (uint32_t)(u >> 32);
  const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0) return 0.f;
  if (e >= 255) return (hi >> 31) ? -3e38f : 3e38f;
  const uint32_t mant = (uint32_t)((u >> 29) & 0x7fffff);
  return __uint_as_float((hi & 0x80000000u) | ((uint32_t)e << 23) | mant);
}

// Bucket coordinate of an in-domain coordinate: FP32 estimate, then the exact
// boundary comparisons (bnd[0] = 0, bnd[v] = ord(b_v), bnd[size+1] = max).
__device__ __forceinline__ uint32_t cell_coord(uint64_t u, int d, const ClParams &P,
                                               const uint64_t *b) {
  const uint64_t o = ord_bits(u);
  const int sz = (int)P.size[d];
  float t = floorf(fmaf(approx_f32(u), P.inv_f[d], P.c_f[d]));
  int v = t < 0.f ? 0 : (t > (float)sz ? sz : (int)t);
  for (int it = 0; it <= sz && v < sz && o >= b[v + 1]; ++it) ++v;
  for (int it = 0; it <= sz && v > 0 && o < b[v]; ++it) --v;
  return (uint32_t)v;
}

template <int DIM>
__global__ void __launch_bounds__(CL_TPB) k_cl_keys(double *__restrict__ pos, int64_t n, ClParams P,
                                                    uint32_t *__restrict__ keys,
                                                    ClHeader *__restrict__ H) {
  __shared__ uint32_t h[CL_MAX_PASSES][CL_RADIX];
  __shared__ uint32_t sdead;
  extern __shared__ uint64_t sbnd[];  // the boundary tables when they fit
  for (int i = threadIdx.x; i < P.npasses * CL_RADIX; i += CL_TPB) (&h[0][0])[i] = 0;
  if (threadIdx.x == 0) sdead = 0;
  const bool shared_tab = P.bnd_total <= CL_BND_SMEM;
  if (shared_tab)
    for (int i = threadIdx.x; i < P.bnd_total; i += CL_TPB) sbnd[i] = P.bnd_all[i];
  __syncthreads();
  const uint64_t *tab = shared_tab ? sbnd : P.bnd_all;
  uint32_t dead = 0, err = 0;
  for (int64_t base = (int64_t)blockIdx.x * CL_KEYS_TILE; base < n;
       base += (int64_t)gridDim.x * CL_KEYS_TILE) {
    constexpr int U = 4;  // particles per thread with their loads in flight together
#pragma unroll 1
    for (int it0 = 0; it0 < CL_KEYS_TILE / CL_TPB; it0 += U) {
      double rr[U][DIM];
#pragma unroll
      for (int j = 0; j < U; ++j) {
        const int64_t i = base + (int64_t)(it0 + j) * CL_TPB + threadIdx.x;
#pragma unroll
        for (int d = 0; d < DIM; ++d) rr[j][d] = i < n ? pos[(int64_t)d * n + i] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < U; ++j) {
        const int64_t i = base + (int64_t)(it0 + j) * CL_TPB + threadIdx.x;
        if (i < n) {
          double *r = rr[j];
          bool alive = true;
          uint32_t key = 0, mult = 1;
#pragma unroll
          for (int d = DIM - 1; d >= 0; --d) {
            uint64_t u = (uint64_t)__double_as_longlong(r[d]);
            uint32_t v = 0;
            const uint32_t hw = (uint32_t)(u >> 32);
            const uint32_t ex = (hw >> 20) & 0x7ffu;
            // fast path: the FP32 value shows the coordinate inside the domain
            // and the FP32 bucket estimate away from a cell boundary by more
            // than its error bound, so both decisions are the FP64 ones
            bool fast = false;
            if (ex - 897u < 254u) {  // a normal FP32 exponent
              const float xf = __uint_as_float((hw & 0x80000000u) |
                                               (((hw & 0x7fffffffu) - (896u << 20)) << 3) |
                                               ((uint32_t)u >> 29));
              if (xf >= P.lo_fast[d] && xf <= P.hi_fast[d]) {
                const float t = fmaf(xf, P.inv_f[d], P.c_f[d]);
                const float vf = floorf(t);
                const float fr = t - vf;
                if (fr >= P.delta_f[d] && fr <= 1.0f - P.delta_f[d]) {
                  v = (uint32_t)(int)vf;
                  fast = true;
                }
              }
            }
            if (fast) {
            } else if (ex == 0x7ffu) {  // !isfinite
              alive = false;
            } else {
              uint64_t o = ord_bits(u);
              bool exact = false;
              if (o < P.olo[d] || o >= P.ohi[d]) {
                if (P.periodic[d]) {
                  // the reference's wrap loops (rare)
                  double x = r[d];
                  const double w = __dsub_rn(P.hi[d], P.lo[d]);
                  int k = 0;
                  while (x < P.lo[d] && k < CL_WRAP_CAP) { x = __dadd_rn(x, w); ++k; }
                  while (x >= P.hi[d] && k < CL_WRAP_CAP) { x = __dsub_rn(x, w); ++k; }
                  if (k >= CL_WRAP_CAP) {
                    err = 2;
                    alive = false;
                  }
                  pos[(int64_t)d * n + i] = x;
                  u = (uint64_t)__double_as_longlong(x);
                  o = ord_bits(u);
                  if (o < P.olo[d] || o >= P.ohi[d]) {
                    // the wrap rounded outside [lo, hi): the reference's formula as is
                    v = (uint32_t)(int)floor(__dmul_rn(__dsub_rn(x, P.lo[d]), P.inv[d]));
                    exact = true;
                  }
                } else {
                  alive = false;
                }
              }
              if (alive && !exact) v = cell_coord(u, d, P, tab + P.bnd_off[d]);
            }
            // collapse_index_vector (src/detail/SpatialUtil.h:49-59): last
            // dimension fastest, unsigned 32-bit arithmetic
            if (d != DIM - 1) mult *= P.size[d + 1];
            key += mult * v;
          }
          if (!alive) {
            key = P.dead_key;
            ++dead;
          }
          keys[i] = key;
          atomicAdd(&h[0][key & (CL_RADIX - 1)], 1u);
          for (int p = 1; p < P.npasses; ++p) atomicAdd(&h[p][(key >> (CL_RB * p)) & (CL_RADIX - 1)], 1u);
        }
      }
    }
  }
  if (err) atomicMax(&H->error, err);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dead += __shfl_xor_sync(0xffffffffu, dead, o);
  if ((threadIdx.x & 31) == 0 && dead) atomicAdd(&sdead, dead);
  __syncthreads();
  uint32_t *part = &H->part[blockIdx.x % CL_HIST_COPIES][0][0];
  for (int i = threadIdx.x; i < P.npasses * CL_RADIX; i += CL_TPB) {
    const uint32_t c = (&h[0][0])[i];
    if (c) atomicAdd(&part[i], c);
  }
  if (threadIdx.x == 0 && sdead) atomicAdd(&H->dead, sdead);
  // the last block to finish sums the copies into the pass histograms
  __threadfence();
  __shared__ uint32_t ticket;
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(&H->blocks_done, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  for (int i = threadIdx.x; i < P.npasses * CL_RADIX; i += CL_TPB) {
    uint32_t t = 0;
    for (int c = 0; c < CL_HIST_COPIES; ++c) t += ((volatile uint32_t *)&H->part[c][0][0])[i];
    (&H->hist[0][0])[i] = t;
  }
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Dynamic shared memory of the sort pass: the tile's keys, values and
// within-warp ranks, the per-warp digit counts and the digit bases.
struct SweepSmem {
  uint32_t key[CL_TILE];
  uint32_t val[CL_TILE];
  uint16_t rank[CL_TILE];
  uint16_t wcount[SW_WARPS][CL_RADIX + 2];  // counts, then offsets, per warp (<= 16384)
  uint32_t dbase[CL_RADIX];
  uint32_t wsum[SW_WARPS + 1];
  uint32_t tile, fail;
};

// One stable LSD pass over the digit (key >> 10 pass) & (CL_RADIX - 1).
// A tile is 16384 keys: warp w of 16 ranks its own 1024 consecutive keys in
// two rounds of 512 (lane l holding keys l, l+32, ... of a round, so the slots
// visit them in input order; __match_any_sync gives the stable rank within
// the warp), staging keys, values and ranks in shared memory.  The tile's
// digit counts are published and prefixed by decoupled look-back over the
// preceding tiles (tiles are claimed in order, so every tile waited on is
// already running), then every key is written to its place.  vals_in ==
// nullptr: the values are the input positions (the first pass).
// Status word of (tile, digit): epoch << 34 | flag << 32 | count.
__global__ void __launch_bounds__(SW_TPB) k_cl_onesweep(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, uint32_t n, int pass,
    unsigned long long *__restrict__ status, uint32_t epoch, ClHeader *__restrict__ H) {
  extern __shared__ __align__(16) unsigned char sweep_raw[];
  SweepSmem &S = *reinterpret_cast<SweepSmem *>(sweep_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int shift = CL_RB * pass;
  if (tid == 0) {
    S.tile = atomicAdd(&H->tile_counter[pass], 1u);
    S.fail = 0;
  }
  for (int i = tid; i < SW_WARPS * (CL_RADIX + 2); i += SW_TPB) (&S.wcount[0][0])[i] = 0;
  // global digit bases: exclusive scan of the pass histogram
  constexpr int DPT = CL_RADIX / SW_TPB;  // digits per thread
  uint32_t g[DPT], gs = 0;
#pragma unroll
  for (int q = 0; q < DPT; ++q) {
    g[q] = H->hist[pass][tid * DPT + q];
    gs += g[q];
  }
  uint32_t incl = gs;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) S.wsum[warp] = incl;
  __syncthreads();
  if (tid == 0) {
    uint32_t run = 0;
    for (int w = 0; w < SW_WARPS; ++w) {
      const uint32_t c = S.wsum[w];
      S.wsum[w] = run;
      run += c;
    }
  }
  __syncthreads();
  {
    uint32_t run = S.wsum[warp] + incl - gs;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
      S.dbase[tid * DPT + q] = run;
      run += g[q];
    }
  }
  const uint32_t tile = S.tile;
  const uint32_t lt_mask = (1u << lane) - 1u;
  constexpr int WCHUNK = CL_TILE / SW_WARPS;  // 1024 keys per warp
  for (int round = 0; round < SW_ROUNDS; ++round) {
    const int lbase = warp * WCHUNK + round * (32 * CL_ITEMS);  // within the tile
    const size_t gbase = (size_t)tile * CL_TILE + lbase;
    uint32_t key[CL_ITEMS], val[CL_ITEMS];
    int dig[CL_ITEMS];
#pragma unroll
    for (int i = 0; i < CL_ITEMS; ++i) {
      const size_t gi = gbase + (size_t)i * 32 + lane;
      if (gi < n) {
        key[i] = keys_in[gi];
        val[i] = vals_in ? vals_in[gi] : (uint32_t)gi;
        dig[i] = (key[i] >> shift) & (CL_RADIX - 1);
      } else {
        key[i] = 0;
        val[i] = 0;
        dig[i] = CL_RADIX;  // sentinel, never written out
      }
    }
#pragma unroll
    for (int i = 0; i < CL_ITEMS; ++i) {
      const uint32_t peers = __match_any_sync(0xffffffffu, dig[i]);
      const int leader = 31 - __clz(peers);
      const uint32_t before = __popc(peers & lt_mask);
      const uint32_t cnt = S.wcount[warp][dig[i]];  // the sentinel column CL_RADIX included
      const int li = lbase + i * 32 + lane;
      S.key[li] = key[i];
      S.val[li] = val[i];
      S.rank[li] = (uint16_t)(cnt + before);
      __syncwarp();
      if (lane == leader) S.wcount[warp][dig[i]] = (uint16_t)(cnt + __popc(peers));
      __syncwarp();
    }
  }
  __syncthreads();
  // per digit: warp prefixes and the tile's count, published for every digit
  // first; then the decoupled look-back over the preceding tiles and the
  // inclusive publication
  const unsigned long long ep = (unsigned long long)epoch << 34;
  uint32_t tcount[DPT];
#pragma unroll
  for (int q = 0; q < DPT; ++q) {
    const int d = tid + q * SW_TPB;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < SW_WARPS; ++w) {
      const uint32_t c = S.wcount[w][d];
      S.wcount[w][d] = (uint16_t)run;
      run += c;
    }
    tcount[q] = run;
    st_release(status + (size_t)tile * CL_RADIX + d, ep | (tile == 0 ? ST_INCL : ST_AGG) | run);
  }
  if (tile > 0) {
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
      const int d = tid + q * SW_TPB;
      uint32_t prefix = 0;
      for (int64_t t = (int64_t)tile - 1; t >= 0; --t) {
        const unsigned long long *pp = status + (size_t)t * CL_RADIX + d;
        unsigned long long st = ld_acquire(pp);
        // bounded wait: 200 ms of the global timer or CL_SPIN_CAP polls, and
        // no wait at all once another tile has given up
        uint32_t spins = 0;
        uint64_t t0 = 0;
        bool gave_up = false;
        while ((st >> 34) != (unsigned long long)epoch || ((st >> 32) & 3ull) == 0ull) {
          if ((++spins & 63u) == 0u) {
            uint64_t now;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
            if (t0 == 0) t0 = now;
            if (now - t0 > 200000000ull || spins >= CL_SPIN_CAP ||
                *(volatile uint32_t *)&H->error != 0u) {
              gave_up = true;
              break;
            }
          }
          st = ld_acquire(pp);
        }
        if (gave_up) {
          atomicExch(&S.fail, 1u);
          atomicMax(&H->error, 1u);
          break;
        }
        prefix += (uint32_t)st;
        if (((st >> 32) & 3ull) == 2ull) break;
      }
      st_release(status + (size_t)tile * CL_RADIX + d, ep | ST_INCL | (uint32_t)(prefix + tcount[q]));
      S.dbase[d] += prefix;
    }
  }
  __syncthreads();
  if (S.fail) return;
  const int nvalid = (int)min((size_t)CL_TILE, (size_t)n - (size_t)tile * CL_TILE);
  // staged key li came from position tile * CL_TILE + li and was ranked by
  // warp li / WCHUNK; keys past n were never staged
  for (int li = tid; li < nvalid; li += SW_TPB) {
    const int w = li / WCHUNK;
    const uint32_t k = S.key[li];
    const int d = (k >> shift) & (CL_RADIX - 1);
    const uint32_t dst = S.dbase[d] + S.wcount[w][d] + S.rank[li];
    keys_out[dst] = k;
    vals_out[dst] = S.val[li];
  }
}

// bucket_begin[c] = lower_bound(keys, c), bucket_end[c] = upper_bound(keys,
// c) over the na sorted alive keys: the boundary before position k (keys
// clamped to ncells, with keys[-1] = -1 and keys[na] = ncells) writes
// bucket_begin for the cells in (prev, cur] and bucket_end for [prev, cur).
__global__ void k_cl_ranges(const uint32_t *__restrict__ keys, const ClHeader *__restrict__ H,
                            uint32_t n, uint32_t ncells, uint32_t *__restrict__ bb,
                            uint32_t *__restrict__ be) {
  const uint32_t na = n - H->dead;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= (int64_t)na;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t prev = k == 0 ? -1 : (int64_t)min(keys[k - 1], ncells);
    const int64_t cur = k == (int64_t)na ? (int64_t)ncells : (int64_t)min(keys[k], ncells);
    for (int64_t c = prev + 1; c <= cur && c < (int64_t)ncells; ++c) bb[c] = (uint32_t)k;
    for (int64_t c = prev < 0 ? 0 : prev; c < cur; ++c) be[c] = (uint32_t)k;
  }
}

__global__ void k_cl_gather(const double *__restrict__ pos_in, int64_t n, int dim,
                            const uint32_t *__restrict__ perm, const ClHeader *__restrict__ H,
                            double *__restrict__ pos_out, const int64_t *__restrict__ ids_in,
                            int64_t *__restrict__ ids_out, const double *__restrict__ s_in,
                            double *__restrict__ s_out) {
  const int64_t na = n - (int64_t)H->dead;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < na;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t i = perm[k];
    for (int d = 0; d < dim; ++d) pos_out[(int64_t)d * na + k] = pos_in[(int64_t)d * n + i];
    ids_out[k] = ids_in[i];
    if (s_in) s_out[k] = s_in[i];
  }
}

// Smallest double x with floor(fl(fl(x - lo) * inv)) >= v, or +inf (as the
// maximum ordered key) when no x below hi reaches v.
uint64_t boundary(double lo, double hi, double inv, int v) {
  auto reaches = [&](double x) { return std::floor((x - lo) * inv) >= (double)v; };
  double x = lo + (double)v / inv;
  if (!(x < hi)) x = std::nextafter(hi, -HUGE_VAL);
  if (x < lo) x = lo;
  int steps = 0;
  while (!reaches(x) && x < hi && steps < (1 << 20)) {
    x = std::nextafter(x, HUGE_VAL);
    ++steps;
  }
  if (!reaches(x) || !(x < hi)) return ~0ull;
  while (x > lo && reaches(std::nextafter(x, -HUGE_VAL)) && steps < (1 << 21)) {
    x = std::nextafter(x, -HUGE_VAL);
    ++steps;
  }
  return ord_host(x);
}

bool same_grid(const GridDesc &a, const GridDesc &b) {
  for (int d = 0; d < 3; ++d)
    if (a.size[d] != b.size[d] || a.side[d] != b.side[d] || a.inv_side[d] != b.inv_side[d] ||
        a.lo[d] != b.lo[d] || a.hi[d] != b.hi[d] || a.periodic[d] != b.periodic[d])
      return false;
  return a.ncells == b.ncells;
}

int run_build(abx_particles *p, const GridDesc &g, uint32_t *dead_out) {
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = p->n;
  const int D = p->dim;
  // cell boundaries of this grid (host, exact), cached with the grid
  if (!p->cl_bnd_valid || !same_grid(p->cl_bnd_grid, g)) {
    std::vector<uint64_t> tab;
    size_t off[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
      off[d] = tab.size();
      const int sz = (int)g.size[d];
      tab.push_back(0ull);
      for (int v = 1; v <= sz; ++v) tab.push_back(boundary(g.lo[d], g.hi[d], g.inv_side[d], v));
      tab.push_back(~0ull);
    }
    ABX_TRY(p->cl_bnd.reserve(tab.size()));
    ABX_CHECK_CUDA(cudaMemcpyAsync(p->cl_bnd.ptr, tab.data(), tab.size() * 8,
                                   cudaMemcpyHostToDevice, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    for (int d = 0; d < 3; ++d) p->cl_bnd_off[d] = off[d];
    p->cl_bnd_grid = g;
    p->cl_bnd_valid = true;
  }
  ClParams P{};
  P.dim = D;
  uint64_t maxkey = 0, mult = 1;
  for (int d = D - 1; d >= 0; --d) {
    if (d != D - 1) mult *= g.size[d + 1];
    maxkey += mult * (uint64_t)g.size[d];
  }
  ABX_REQUIRE(maxkey + 1 <= 0xFFFFFFFFull, ABX_ERR_INVALID, "cell grid too large for 32-bit keys");
  P.dead_key = (uint32_t)(maxkey + 1);
  int bits = 0;
  while (bits < 32 && ((uint64_t)P.dead_key >> bits) != 0) ++bits;
  P.npasses = (bits + CL_RB - 1) / CL_RB;
  if (P.npasses < 1) P.npasses = 1;
  for (int d = 0; d < 3; ++d) {
    P.size[d] = g.size[d];
    P.lo[d] = g.lo[d];
    P.hi[d] = g.hi[d];
    P.inv[d] = g.inv_side[d];
    P.periodic[d] = g.periodic[d];
    P.olo[d] = ord_host(g.lo[d]);
    P.ohi[d] = ord_host(g.hi[d]);
    P.inv_f[d] = (float)g.inv_side[d];
    P.c_f[d] = (float)(-g.lo[d] * g.inv_side[d]);
    // with M = max |bound|: the FP32 value xf of an in-range x (mantissa
    // truncated) is within M 2^-23 of x, so xf in [lo_fast, hi_fast] (lo + m
    // and hi - m rounded inwards, m = M 2^-21) puts x inside [lo, hi); the
    // FP32 estimate of (x - lo) inv is then within M inv 2^-21 + (size+1)
    // 2^-23 of the FP64 one, delta_f doubles that
    const double M = std::max(std::fabs(g.lo[d]), std::fabs(g.hi[d]));
    const double m = std::ldexp(M, -21);
    P.lo_fast[d] = std::nextafter((float)(g.lo[d] + m), HUGE_VALF);
    P.hi_fast[d] = std::nextafter((float)(g.hi[d] - m), -HUGE_VALF);
    P.delta_f[d] = (float)(std::ldexp(M * g.inv_side[d], -20) +
                           std::ldexp((double)g.size[d] + 2.0, -22) + 1e-7);
    if (!(P.delta_f[d] < 0.25f) || !(P.lo_fast[d] < P.hi_fast[d])) {
      // cells too fine for the FP32 estimate: every coordinate takes the exact path
      P.lo_fast[d] = HUGE_VALF;
      P.hi_fast[d] = -HUGE_VALF;
    }
    P.bnd[d] = p->cl_bnd.ptr + p->cl_bnd_off[d];
    P.bnd_off[d] = (int)p->cl_bnd_off[d];
  }
  P.bnd_all = p->cl_bnd.ptr;
  P.bnd_total = 0;
  for (int d = 0; d < D; ++d) P.bnd_total += (int)g.size[d] + 2;
  const size_t keys_smem = P.bnd_total <= CL_BND_SMEM ? (size_t)P.bnd_total * 8 : 0;
  const int ntiles = (int)((n + CL_TILE - 1) / CL_TILE);
  // scratch: header, vals, keys_alt, vals_alt
  size_t o = 0;
  carve_size<ClHeader>(o, 1);
  carve_size<uint32_t>(o, n);
  carve_size<uint32_t>(o, n);
  carve_size<uint32_t>(o, n);
  ABX_TRY(ctx->scratch.reserve(o + 256));
  unsigned char *sb = ctx->scratch.ptr;
  o = 0;
  ClHeader *H = carve<ClHeader>(sb, o, 1);
  uint32_t *vals = carve<uint32_t>(sb, o, n);
  uint32_t *keys_alt = carve<uint32_t>(sb, o, n);
  uint32_t *vals_alt = carve<uint32_t>(sb, o, n);
  ABX_TRY(p->keys.reserve(n));
  const size_t nstatus = (size_t)ntiles * CL_RADIX;
  if (p->cl_status.cap < nstatus) {
    ABX_TRY(p->cl_status.reserve(nstatus));
    ABX_CHECK_CUDA(cudaMemsetAsync(p->cl_status.ptr, 0, nstatus * 8, s));
  }
  ABX_CHECK_CUDA(cudaMemsetAsync(H, 0, sizeof(ClHeader), s));
  ABX_CHECK_CUDA(cudaFuncSetAttribute(k_cl_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(SweepSmem)));
  const int kblocks = (int)std::min<int64_t>((n + CL_KEYS_TILE - 1) / CL_KEYS_TILE,
                                             (int64_t)ctx->num_sms * 4);
  if (D == 1)
    k_cl_keys<1><<<kblocks, CL_TPB, keys_smem, s>>>(p->pos.ptr, n, P, p->keys.ptr, H);
  else if (D == 2)
    k_cl_keys<2><<<kblocks, CL_TPB, keys_smem, s>>>(p->pos.ptr, n, P, p->keys.ptr, H);
  else
    k_cl_keys<3><<<kblocks, CL_TPB, keys_smem, s>>>(p->pos.ptr, n, P, p->keys.ptr, H);
  ABX_CHECK_CUDA(cudaGetLastError());
  uint32_t *ki = p->keys.ptr, *vi = nullptr, *ko = keys_alt, *vo = vals;
  for (int pass = 0; pass < P.npasses; ++pass) {
    p->cl_epoch = (p->cl_epoch + 1) & 0x3fffffffu;
    if (p->cl_epoch == 0) p->cl_epoch = 1;
    k_cl_onesweep<<<ntiles, SW_TPB, sizeof(SweepSmem), s>>>(ki, vi, ko, vo, (uint32_t)n, pass,
                                                            p->cl_status.ptr, p->cl_epoch, H);
    if (pass == 0) vi = vals_alt;
    ABX_CHECK_CUDA(cudaGetLastError());
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  if (ki != p->keys.ptr)
    ABX_CHECK_CUDA(cudaMemcpyAsync(p->keys.ptr, ki, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
  ABX_TRY(p->bucket_begin.reserve(g.ncells));
  ABX_TRY(p->bucket_end.reserve(g.ncells));
  const int rblocks = (int)std::min<int64_t>((n + 1 + 255) / 256, (int64_t)ctx->num_sms * 16);
  k_cl_ranges<<<rblocks, 256, 0, s>>>(p->keys.ptr, H, (uint32_t)n, g.ncells, p->bucket_begin.ptr,
                                      p->bucket_end.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_TRY(p->pos_alt.reserve((size_t)D * n));
  ABX_TRY(p->ids_alt.reserve(n));
  if (p->has_scalar) ABX_TRY(p->scalar_alt.reserve(n));
  const int gblocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 16);
  k_cl_gather<<<gblocks, 256, 0, s>>>(p->pos.ptr, n, D, vi, H, p->pos_alt.ptr, p->ids.ptr,
                                      p->ids_alt.ptr, p->has_scalar ? p->scalar.ptr : nullptr,
                                      p->has_scalar ? p->scalar_alt.ptr : nullptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  uint32_t hd[2];
  ABX_CHECK_CUDA(cudaMemcpyAsync(hd, &H->dead, 8, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  ABX_REQUIRE(hd[1] != 1, ABX_ERR_TIMEOUT, "cell-list sort: a look-back wait gave up");
  ABX_REQUIRE(hd[1] != 2, ABX_ERR_INVALID,
              "a periodic coordinate too far outside the domain to wrap back");
  *dead_out = hd[0];
  return ABX_OK;
}

}  // namespace

// GridDesc that set_domain_impl would leave for alive count n, and the count
// it would record, without changing the particle set.
GridDesc grid_for_count(const abx_particles *p, size_t n, size_t *calc_n);

int celllist_build(abx_particles *p) {
  const int64_t n = p->n;
  ABX_REQUIRE(n < ((int64_t)1 << 30), ABX_ERR_INVALID, "too many particles for the cell list (%lld)",
              (long long)n);
  size_t calc_all = 0, calc_alive = 0;
  const GridDesc g_all = grid_for_count(p, (size_t)n, &calc_all);
  uint32_t dead = 0;
  ABX_TRY(run_build(p, g_all, &dead));
  const int64_t na = n - (int64_t)dead;
  GridDesc g = grid_for_count(p, (size_t)na, &calc_alive);
  if (!same_grid(g, g_all)) {
    // deletions changed the grid: the positions are now enforced in place,
    // so a second build sees the same alive set
    ABX_TRY(run_build(p, g, &dead));
    ABX_REQUIRE(n - (int64_t)dead == na, ABX_ERR_STATE, "alive count changed between builds");
  }
  p->grid = g;
  p->size_calculated_with_n = calc_alive;
  std::swap(p->pos.ptr, p->pos_alt.ptr);
  std::swap(p->pos.cap, p->pos_alt.cap);
  std::swap(p->ids.ptr, p->ids_alt.ptr);
  std::swap(p->ids.cap, p->ids_alt.cap);
  if (p->has_scalar) {
    std::swap(p->scalar.ptr, p->scalar_alt.ptr);
    std::swap(p->scalar.cap, p->scalar_alt.cap);
  }
  p->n = na;
  p->n_alive_prev = na;
  return ABX_OK;
}

}  // namespace abx
