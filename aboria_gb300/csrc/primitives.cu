// Device primitives for the cell-list build: exclusive scan and a stable LSD
// radix sort of (u32 key, u32 value) pairs.
//
// The reference reaches these through Thrust (detail::exclusive_scan,
// detail::sort_by_key: src/detail/Algorithms.h:173-206, :551-580).  Its Thrust
// backend sorts stably (thrust::sort_by_key, :195), which is the order this
// sort reproduces: (key, input position).
//
// Layout: tiles of 4096 items (256 threads x 16).  Within a tile each warp owns
// 512 consecutive items, lane l holding items l, l+32, ... so that walking the
// 16 slots in order visits the warp's items in input order; ranking with
// __match_any_sync then gives a stable per-warp rank without a block-wide
// local sort.
#include "common.cuh"

namespace abx {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive scan of a 4096-item tile held in shared memory; returns the tile
// total to every thread.
__device__ uint32_t block_scan_tile(uint32_t *s, uint32_t *warp_tot) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t local[SCAN_ITEMS];
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    local[i] = s[tid * SCAN_ITEMS + i];
    sum += local[i];
  }
  uint32_t incl = warp_incl_scan(sum);
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (SCAN_THREADS / 32) ? warp_tot[lane] : 0;
    uint32_t wi = warp_incl_scan(w);
    if (lane < (SCAN_THREADS / 32)) warp_tot[lane] = wi - w;
    if (lane == (SCAN_THREADS / 32) - 1) warp_tot[SCAN_THREADS / 32] = wi;
  }
  __syncthreads();
  uint32_t run = warp_tot[warp] + incl - sum;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    s[tid * SCAN_ITEMS + i] = run;
    run += local[i];
  }
  uint32_t total = warp_tot[SCAN_THREADS / 32];
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t *in, size_t n,
                                                              uint32_t *block_sums) {
  __shared__ uint32_t red[SCAN_THREADS / 32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  uint32_t sum = 0;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    size_t g = base + i;
    if (g < n) sum += in[g];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < SCAN_THREADS / 32; ++w) t += red[w];
    block_sums[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(uint32_t *data, size_t n,
                                                             const uint32_t *block_offsets) {
  __shared__ uint32_t s[SCAN_TILE];
  __shared__ uint32_t warp_tot[SCAN_THREADS / 32 + 1];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    size_t g = base + i;
    s[i] = g < n ? data[g] : 0u;
  }
  __syncthreads();
  block_scan_tile(s, warp_tot);
  const uint32_t off = block_offsets ? block_offsets[blockIdx.x] : 0u;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    size_t g = base + i;
    if (g < n) data[g] = s[i] + off;
  }
}

// ---------------------------------------------------------------- radix ---
// LSD radix sort of (key, value) pairs, stable; RB-bit digits (8, or 10 when
// two 10-bit passes cover the key where 8-bit digits would need three).
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // 4096
constexpr int RADIX_MAX = 1 << 10;

template <int RB>
__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(const uint32_t *keys, size_t n,
                                                           int shift, uint32_t mask,
                                                           uint32_t *hist, int ntiles) {
  constexpr int RADIX = 1 << RB;
  __shared__ uint32_t h[RADIX];
  for (int i = threadIdx.x; i < RADIX; i += RS_THREADS) h[i] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * RS_TILE;
  for (int i = threadIdx.x; i < RS_TILE; i += RS_THREADS) {
    size_t g = base + i;
    if (g < n) atomicAdd(&h[(keys[g] >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += RS_THREADS)
    hist[(size_t)d * ntiles + blockIdx.x] = h[d];
}

template <int RB>
__global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, size_t n, int shift,
    uint32_t mask, const uint32_t *__restrict__ offsets, int ntiles) {
  constexpr int RADIX = 1 << RB;
  __shared__ uint32_t wcount[RS_WARPS][RADIX + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < RS_WARPS * (RADIX + 1); i += RS_THREADS) (&wcount[0][0])[i] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)warp * (32 * RS_ITEMS);
  uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
  int dig[RS_ITEMS];
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int i = 0; i < RS_ITEMS; ++i) {
    size_t g = base + (size_t)i * 32 + lane;
    if (g < n) {
      key[i] = keys_in[g];
      val[i] = vals_in[g];
      dig[i] = (key[i] >> shift) & mask;
    } else {
      key[i] = 0;
      val[i] = 0;
      dig[i] = RADIX;  // sentinel bucket, never written out
    }
  }
#pragma unroll
  for (int i = 0; i < RS_ITEMS; ++i) {
    const uint32_t peers = __match_any_sync(0xffffffffu, dig[i]);
    const int leader = 31 - __clz(peers);
    const uint32_t before = __popc(peers & lt_mask);
    const uint32_t cnt = wcount[warp][dig[i]];
    rank[i] = cnt + before;
    __syncwarp();
    if (lane == leader) wcount[warp][dig[i]] = cnt + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive prefix over warps, per digit
  for (int d = tid; d < RADIX; d += RS_THREADS) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < RS_ITEMS; ++i) {
    if (dig[i] < RADIX) {
      const size_t dst = (size_t)offsets[(size_t)dig[i] * ntiles + blockIdx.x] +
                         wcount[warp][dig[i]] + rank[i];
      keys_out[dst] = key[i];
      vals_out[dst] = val[i];
    }
  }
}

}  // namespace

size_t scan_temp_elems(size_t n) {
  size_t total = 0;
  size_t m = n;
  while (m > (size_t)SCAN_TILE) {
    m = (m + SCAN_TILE - 1) / SCAN_TILE;
    total += m + 64;  // padding keeps levels apart
  }
  return total + 64;
}

int exclusive_scan_u32(uint32_t *data, size_t n, uint32_t *temp, cudaStream_t s) {
  if (n == 0) return ABX_OK;
  if (n <= (size_t)SCAN_TILE) {
    k_scan_tiles<<<1, SCAN_THREADS, 0, s>>>(data, n, nullptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    return ABX_OK;
  }
  const size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  uint32_t *sums = temp;
  k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(data, n, sums);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_TRY(exclusive_scan_u32(sums, nb, temp + nb + 64, s));
  k_scan_tiles<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(data, n, sums);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

size_t radix_temp_u32(size_t n) {
  const size_t ntiles = (n + RS_TILE - 1) / RS_TILE;
  const size_t hist = ntiles * RADIX_MAX;
  return hist + 64 + scan_temp_elems(hist);
}

int radix_sort_pairs(uint32_t *keys, uint32_t *vals, size_t n, int bits, uint32_t *keys_alt,
                     uint32_t *vals_alt, uint32_t *temp, cudaStream_t s) {
  if (n <= 1 || bits <= 0) return ABX_OK;
  // digit width: 10 bits where that saves a pass (17..20-bit keys)
  const int rb = (bits > 16 && bits <= 20) ? 10 : 8;
  const int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
  const size_t hist_n = (size_t)ntiles << rb;
  uint32_t *hist = temp;
  uint32_t *scan_tmp = temp + hist_n + 64;
  uint32_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
  for (int shift = 0; shift < bits; shift += rb) {
    const int nb = bits - shift < rb ? bits - shift : rb;
    const uint32_t mask = (1u << nb) - 1u;
    if (rb == 10)
      k_radix_hist<10><<<ntiles, RS_THREADS, 0, s>>>(ki, n, shift, mask, hist, ntiles);
    else
      k_radix_hist<8><<<ntiles, RS_THREADS, 0, s>>>(ki, n, shift, mask, hist, ntiles);
    ABX_CHECK_CUDA(cudaGetLastError());
    ABX_TRY(exclusive_scan_u32(hist, hist_n, scan_tmp, s));
    if (rb == 10)
      k_radix_scatter<10><<<ntiles, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, mask, hist, ntiles);
    else
      k_radix_scatter<8><<<ntiles, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, mask, hist, ntiles);
    ABX_CHECK_CUDA(cudaGetLastError());
    uint32_t *t;
    t = ki; ki = ko; ko = t;
    t = vi; vi = vo; vo = t;
  }
  if (ki != keys) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(keys, ki, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    ABX_CHECK_CUDA(cudaMemcpyAsync(vals, vi, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
  return ABX_OK;
}

}  // namespace abx
