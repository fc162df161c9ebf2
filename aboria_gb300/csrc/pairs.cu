// Radius search and the matrix-free sparse operator on the GPU.
//
// Reference path restated: KernelSparse::evaluate (src/Kernels.h:720-751)
// calls euclidean_search (src/Search.h:839-845) per row, which walks periodic
// images x buckets of the CellListOrdered grid and accepts a candidate iff
// !(((0+dx0^2)+dx1^2)+dx2^2 > r^2) in FP64 with dx = x_j - (x_i + image*L)
// (src/Search.h:438-465, src/detail/Distance.h:132-137); it then accumulates
// c_i += f(dx, a_i, b_j) * b_j.
//
// GB300 design (not a translation of the bucket-walk iterator):
//  * An internal fine grid of side ~r/3 (padded to 3 dims, last real
//    dimension fastest) re-sorts the column particles so that each (e0,e1)
//    row of fine cells is one contiguous index range; a query tile then
//    visits ~49 contiguous ranges instead of iterating buckets.
//  * Work unit = one warp = up to 32 spatially adjacent queries.  The warp
//    stages 32 candidates at a time in shared memory (one coalesced 16 B load
//    per lane) and every lane tests its query against all of them
//    (broadcast LDS), so each candidate costs one LDS + the pair arithmetic.
//  * Mixed mode: candidate and query coordinates are FP32 offsets from the
//    tile's reference cell (magnitude <= a few cells, so ~1e-9 absolute
//    error).  A pair is accepted outright if d2 <= r2_lo, rejected if
//    d2 > r2_hi, and only inside that rounding band is the reference's exact
//    FP64 test evaluated, so neighbour decisions are identical to the FP64
//    test.  Kernel values are FP32; each lane sums a staged block of <= 32
//    terms in FP32 and adds the block into an FP64 accumulator.
//  * FP64 mode: candidates are staged as absolute FP64 positions and every
//    pair evaluates the reference's formula exactly (no FMA contraction).
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "handles.cuh"

namespace abx {

struct alignas(32) D4 {
  double x, y, z, w;
};

struct FineGrid {
  int dim, eoff;
  int m[3];
  double h[3];
  float hf[3];
  double lo[3];
  double L[3];
  int periodic[3];
  int K[3];
  uint32_t ncells;
};

// A point set ordered by fine cell.
struct PointLayout {
  int64_t n = 0;
  DevBuf<uint32_t> perm;  // kernel order -> source index
  DevBuf<int4> cell;      // unclamped fine cell (internal dims)
  DevBuf<float4> loc;     // FP32 offset from the clamped cell corner; .w = clamped c2 bits
  DevBuf<D4> posk;        // FP64 position in kernel order (internal dims, pad = 0)
  DevBuf<uint32_t> keys;  // sorted clamped cell keys
};

struct PairLayout {
  FineGrid fg;
  double r = 0;
  uint64_t cols_version = 0, rows_version = 0;
  bool self = true;
  PointLayout cols;
  PointLayout rows_own;
  PointLayout *rows = nullptr;
  DevBuf<uint32_t> cell_start;  // fg.ncells + 1
  DevBuf<int2> units;           // (first query in kernel order, count <= 32)
  int nunits = 0;
  DevBuf<float> bk32;
  DevBuf<double> bk64;
  DevBuf<double> sk;  // column scalar in kernel order
  DevBuf<double> sq;  // row scalar in kernel order
  DevBuf<double> ck;  // result in row kernel order
  DevBuf<int> counter;
  DevBuf<int> ext;  // e2 extent table
};

void pair_layout_free(PairLayout *L) { delete L; }

namespace {

constexpr int TPB = 256;
constexpr int WARPS_PER_CTA = 4;
constexpr int GROUP_E2 = 4;  // a unit spans at most this many fine cells along e2

enum { POL_COUNT = 0, POL_LIST = 1, POL_MATVEC = 2 };

// ------------------------------------------------------------ layout build ---
FineGrid make_fine_grid(const GridDesc &g, double r, int64_t npts, int F) {
  FineGrid fg{};
  fg.dim = g.dim;
  fg.eoff = 3 - g.dim;
  const double target = r > 0 ? r / F : 0.0;
  for (int e = 0; e < 3; ++e) {
    const int d = e - fg.eoff;
    if (d < 0) {
      fg.m[e] = 1;
      fg.h[e] = 1.0;
      fg.lo[e] = 0.0;
      fg.L[e] = 1.0;
      fg.periodic[e] = 0;
      continue;
    }
    fg.lo[e] = g.lo[d];
    fg.L[e] = g.hi[d] - g.lo[d];
    fg.periodic[e] = g.periodic[d];
    double m = target > 0 ? std::floor(fg.L[e] / target * (1.0 - 1e-9)) : 1.0;
    if (!(m >= 1.0)) m = 1.0;
    if (m > 1023.0) m = 1023.0;
    fg.m[e] = (int)m;
  }
  // keep the fine grid within a few cells per point
  const double cap = std::max<double>(64.0, 4.0 * (double)npts);
  for (int it = 0; it < 64; ++it) {
    double tot = (double)fg.m[0] * fg.m[1] * fg.m[2];
    if (tot <= cap) break;
    int eb = 0;
    for (int e = 1; e < 3; ++e)
      if (fg.m[e] > fg.m[eb]) eb = e;
    fg.m[eb] = std::max(1, (int)(fg.m[eb] * 0.8));
  }
  fg.ncells = (uint32_t)fg.m[0] * fg.m[1] * fg.m[2];
  for (int e = 0; e < 3; ++e) {
    const int d = e - fg.eoff;
    fg.h[e] = d < 0 ? 1.0 : fg.L[e] / fg.m[e];
    fg.hf[e] = (float)fg.h[e];
    fg.K[e] = d < 0 ? 0 : (int)std::ceil(r / fg.h[e] * (1.0 + 1e-9));
    if (fg.K[e] > 2 * fg.m[e] + 1) fg.K[e] = 2 * fg.m[e] + 1;
  }
  return fg;
}

__device__ __forceinline__ int fine_coord(double x, double lo, double h, int m) {
  // floor((x - lo)/h) computed as in the layout; unclamped
  const double t = floor((x - lo) / h);
  if (!(t == t)) return 1000000000;  // NaN: far outside, never a neighbour
  if (t < -1e9) return -1000000000;
  if (t > 1e9) return 1000000000;
  return (int)t;
}

// Sort key of a point: clamped fine cell (row-major, e2 fastest) times 8 plus
// its octant within the cell, so that consecutive points of a dense cell are
// also close together (tighter query tiles).
__global__ void k_fine_keys(const double *__restrict__ src, int64_t n, int64_t stride, FineGrid fg,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  uint32_t sub = 0;
  for (int e = 0; e < 3; ++e) {
    const int d = e - fg.eoff;
    if (d < 0) {
      c[e] = 0;
      continue;
    }
    const double x = src[(int64_t)d * stride + i];
    int u = fine_coord(x, fg.lo[e], fg.h[e], fg.m[e]);
    c[e] = min(max(u, 0), fg.m[e] - 1);
    const double f = x - (fg.lo[e] + (double)c[e] * fg.h[e]);
    sub |= (f >= 0.5 * fg.h[e] ? 1u : 0u) << (2 - e);
  }
  keys[i] = ((((uint32_t)c[0] * fg.m[1] + c[1]) * fg.m[2] + c[2]) << 3) | sub;
  vals[i] = (uint32_t)i;
}

// Anchor cell of a point: the clamped cell for column particles (their range
// membership), the unclamped cell for query points (which may lie outside
// the domain and must keep their true periodic image).  loc holds the FP32
// offset from the anchor cell's corner and, in .w, the anchor's e2 index as
// an (exact) float.
__global__ void k_fill_layout(const double *__restrict__ src, int64_t stride, FineGrid fg,
                              const uint32_t *__restrict__ perm, int64_t n, int clamp_anchor,
                              int4 *__restrict__ cell, float4 *__restrict__ loc,
                              D4 *__restrict__ posk) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = perm[k];
  double x[3];
  int u[3], c[3];
  float f[3];
  for (int e = 0; e < 3; ++e) {
    const int d = e - fg.eoff;
    if (d < 0) {
      x[e] = 0.0;
      u[e] = 0;
      c[e] = 0;
      f[e] = 0.f;
      continue;
    }
    x[e] = src[(int64_t)d * stride + i];
    u[e] = fine_coord(x[e], fg.lo[e], fg.h[e], fg.m[e]);
    c[e] = clamp_anchor ? min(max(u[e], 0), fg.m[e] - 1) : u[e];
    const double corner = fg.lo[e] + (double)c[e] * fg.h[e];
    f[e] = (float)(x[e] - corner);
  }
  cell[k] = make_int4(c[0], c[1], c[2], 0);
  loc[k] = make_float4(f[0], f[1], f[2], (float)c[2]);  // exact: c[2] < 2^24
  posk[k] = D4{x[0], x[1], x[2], 0.0};
}

__global__ void k_mark_runs_fine(const uint32_t *__restrict__ keys, int64_t n,
                                 uint32_t *__restrict__ first, uint32_t *__restrict__ last) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t key = keys[k] >> 3;
  if (k == 0 || (keys[k - 1] >> 3) != key) first[key] = (uint32_t)k;
  if (k == n - 1 || (keys[k + 1] >> 3) != key) last[key] = (uint32_t)(k + 1);
}

__global__ void k_sub(const uint32_t *__restrict__ a, uint32_t n, uint32_t *__restrict__ b) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) b[c] -= a[c];
}

int build_points(abx_context *ctx, const double *src_soa, int64_t n, int64_t stride,
                 const FineGrid &fg, bool clamp_anchor, PointLayout &P) {
  cudaStream_t s = ctx->stream;
  P.n = n;
  ABX_TRY(P.perm.reserve(n ? n : 1));
  ABX_TRY(P.keys.reserve(n ? n : 1));
  ABX_TRY(P.cell.reserve(n ? n : 1));
  ABX_TRY(P.loc.reserve(n ? n : 1));
  ABX_TRY(P.posk.reserve(n ? n : 1));
  if (n == 0) return ABX_OK;
  DevBuf<uint32_t> tmp;
  const size_t rt = radix_temp_u32(n);
  ABX_TRY(tmp.reserve(2 * (size_t)n + rt + 64));
  k_fine_keys<<<ceil_div(n, TPB), TPB, 0, s>>>(src_soa, n, stride, fg, P.keys.ptr, P.perm.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  int bits = 0;
  while (bits < 32 && (((uint64_t)fg.ncells * 8 - 1) >> bits) != 0) ++bits;
  ABX_TRY(radix_sort_pairs(P.keys.ptr, P.perm.ptr, n, bits, tmp.ptr, tmp.ptr + n, tmp.ptr + 2 * n,
                           s));
  k_fill_layout<<<ceil_div(n, TPB), TPB, 0, s>>>(src_soa, stride, fg, P.perm.ptr, n,
                                                 clamp_anchor ? 1 : 0, P.cell.ptr, P.loc.ptr,
                                                 P.posk.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

int build_cell_start(abx_context *ctx, PairLayout &L) {
  cudaStream_t s = ctx->stream;
  const uint32_t nc = L.fg.ncells;
  ABX_TRY(L.cell_start.reserve((size_t)nc + 1));
  DevBuf<uint32_t> first;
  ABX_TRY(first.reserve((size_t)nc + 1 + scan_temp_elems((size_t)nc + 1)));
  uint32_t *cs = L.cell_start.ptr;
  ABX_CHECK_CUDA(cudaMemsetAsync(cs, 0, ((size_t)nc + 1) * 4, s));
  ABX_CHECK_CUDA(cudaMemsetAsync(first.ptr, 0, ((size_t)nc + 1) * 4, s));
  const int64_t n = L.cols.n;
  if (n > 0) {
    k_mark_runs_fine<<<ceil_div(n, TPB), TPB, 0, s>>>(L.cols.keys.ptr, n, first.ptr, cs);
    ABX_CHECK_CUDA(cudaGetLastError());
    k_sub<<<ceil_div(nc, TPB), TPB, 0, s>>>(first.ptr, nc, cs);
    ABX_CHECK_CUDA(cudaGetLastError());
  }
  // counts -> exclusive scan over nc+1 entries (last entry 0 -> total)
  ABX_TRY(exclusive_scan_u32(cs, (size_t)nc + 1, first.ptr + nc + 1, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

// Units: greedy runs of <= 32 consecutive queries (kernel order) whose anchor
// cells share (e0, e1) and span fewer than GROUP_E2 cells along e2.
int build_units(abx_context *ctx, PairLayout &L) {
  PointLayout &Q = *L.rows;
  const int64_t n = Q.n;
  ABX_REQUIRE(n < (int64_t)0x7fffffff, ABX_ERR_INVALID, "too many query points");
  std::vector<int4> cell(n);
  if (n) ABX_CHECK_CUDA(cudaMemcpy(cell.data(), Q.cell.ptr, n * sizeof(int4), cudaMemcpyDeviceToHost));
  std::vector<int2> units;
  units.reserve(n / 16 + 16);
  int64_t i = 0;
  while (i < n) {
    const int4 c0 = cell[i];
    int zmin = c0.z, zmax = c0.z;
    int64_t j = i + 1;
    while (j < n && j - i < 32) {
      const int4 cj = cell[j];
      if (cj.x != c0.x || cj.y != c0.y) break;
      const int nz0 = std::min(zmin, cj.z), nz1 = std::max(zmax, cj.z);
      if (nz1 - nz0 >= GROUP_E2) break;
      zmin = nz0;
      zmax = nz1;
      ++j;
    }
    units.push_back(make_int2((int)i, (int)(j - i)));
    i = j;
  }
  L.nunits = (int)units.size();
  ABX_TRY(L.units.reserve(units.size() ? units.size() : 1));
  if (!units.empty())
    ABX_CHECK_CUDA(cudaMemcpy(L.units.ptr, units.data(), units.size() * sizeof(int2),
                              cudaMemcpyHostToDevice));
  ABX_TRY(L.counter.reserve(4));
  return ABX_OK;
}

// ------------------------------------------------------------- kernels ---
constexpr int EXT_TAB = 64;   // extent table covers gaps of < 64 cells in e0, e1
constexpr int SEG_CAP = 96;   // segments per batch (32 rows x up to 3 image splits)

struct KParams {
  FineGrid fg;
  double r, r2;
  double prune2;  // squared pruning distance (r plus a safety margin)
  // radius-search norm: 2 euclidean, 1 manhattan, -1 chebyshev (the
  // reference's distance_helper<2/1/-1>); thr = get_value_to_accumulate(r)
  int lnorm;
  double thr;
  const int *ext;  // [EXT_TAB*EXT_TAB]: max e2 gap (cells) for e0/e1 gaps, -1 pruned
  // kernel functor parameters
  int kind;
  double p0;
  float p0f, c_exp2;  // c_exp2 = -p0*log2(e)
  // columns (kernel order)
  const float4 *cloc;
  const D4 *cpos;
  const uint32_t *cell_start;
  const float *b32;
  const double *b64;
  const double *s_col;
  // queries (kernel order)
  const int4 *qcell;
  const float4 *qloc;
  const D4 *qpos;
  const double *s_row;
  const int2 *units;
  int nunits;
  int *counter;
  // outputs (query kernel order)
  int32_t *counts;
  const int64_t *rowptr;  // for LIST: query kernel order -> output offset
  int32_t *cols_out;      // storage index of the column particle
  double *dx_out;         // for LIST (optional): x_j - (x_i + image*L), D per pair
  const uint32_t *cperm;  // column kernel order -> storage index
  double *c;
};

// Hardware base-2 exponential (MUFU, ~2 ulp), flush-to-zero: the kernel
// weights it serves are negligible long before 2^-126.
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <int KIND> __device__ __forceinline__ float kern32(float d2, const KParams &P) {
  if (KIND == ABX_K_CONST) return P.p0f;
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return ex2_approx(d2 * P.c_exp2);
  if (KIND == ABX_K_WENDLAND_C2) {
    const float q = d2 * rsqrtf(fmaxf(d2, 1e-36f)) * P.p0f;
    const float t = fmaxf(1.0f - q, 0.0f);
    const float t2 = t * t;
    return t2 * t2 * fmaf(4.0f, q, 1.0f);
  }
  if (KIND == ABX_K_LAPLACE) return __fdividef(1.0f, d2 * rsqrtf(fmaxf(d2, 1e-36f)) + P.p0f);
  if (KIND == ABX_K_MULTIQUADRIC) {
    const float a = d2 + P.p0f;
    return a * rsqrtf(fmaxf(a, 1e-36f));
  }
  return 0.f;
}

template <int KIND>
__device__ __forceinline__ double kern64(double d2, const KParams &P, double si, double sj) {
  if (KIND == ABX_K_CONST) return P.p0;
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return exp(-d2 * P.p0);
  if (KIND == ABX_K_WENDLAND_C2) {
    const double q = sqrt(d2) * P.p0;
    if (q >= 1.0) return 0.0;
    const double t = 1.0 - q;
    const double t2 = t * t;
    return t2 * t2 * (4.0 * q + 1.0);
  }
  if (KIND == ABX_K_LAPLACE) return 1.0 / (sqrt(d2) + P.p0);
  if (KIND == ABX_K_MULTIQUADRIC) return sqrt(d2 + P.p0);
  if (KIND == ABX_K_SCALAR_SUM) return si + sj;
  return 0.0;
}

// The reference's FP64 acceptance test for one (query, candidate, image):
// accum = ((0 + dx0^2) + dx1^2) + dx2^2 over the REAL dimensions in order, no
// FMA, with dx = x_j - (x_i + image*L); inside iff !(accum > r^2).
__device__ __forceinline__ double exact_d2(const D4 &xq, const D4 &xj, const int *img,
                                           const FineGrid &fg) {
  const double q[3] = {xq.x, xq.y, xq.z};
  const double p[3] = {xj.x, xj.y, xj.z};
  double acc = 0.0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e < fg.eoff) continue;
    const double cur = __dadd_rn(q[e], __dmul_rn((double)img[e], fg.L[e]));
    const double dx = __dsub_rn(p[e], cur);
    acc = __dadd_rn(acc, __dmul_rn(dx, dx));
  }
  return acc;
}

// The reference's test in the manhattan and chebyshev norms
// (distance_helper<1>, <-1>, src/detail/Distance.h:46-137): accum starts at 0
// and takes |dx| over the real dimensions in order, summed (1) or as a running
// maximum (-1); inside iff !(accum > |r|).
__device__ __forceinline__ double exact_norm(const D4 &xq, const D4 &xj, const int *img,
                                             const FineGrid &fg, int lnorm) {
  if (lnorm == 2) return exact_d2(xq, xj, img, fg);
  const double q[3] = {xq.x, xq.y, xq.z};
  const double p[3] = {xj.x, xj.y, xj.z};
  double acc = 0.0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e < fg.eoff) continue;
    const double cur = __dadd_rn(q[e], __dmul_rn((double)img[e], fg.L[e]));
    const double a = fabs(__dsub_rn(p[e], cur));
    if (lnorm == 1)
      acc = __dadd_rn(acc, a);
    else if (a > acc)
      acc = a;
  }
  return acc;
}

__device__ __forceinline__ void unpack_seg(int z, int img[3], int &du0, int &du1) {
  img[0] = (z & 3) - 1;
  img[1] = ((z >> 2) & 3) - 1;
  img[2] = ((z >> 4) & 3) - 1;
  du0 = ((z >> 6) & 0xfff) - 2048;
  du1 = ((z >> 18) & 0xfff) - 2048;
}

// dx of an accepted pair as the reference's search iterator exposes it:
// x_j - (x_i + image*L) over the real dimensions (src/Search.h:188-190, 443),
// written as D doubles at pair slot `slot`.
__device__ __forceinline__ void write_dx(const KParams &P, int64_t slot, const D4 &xq, int k,
                                         int seg_z) {
  const FineGrid &fg = P.fg;
  int img[3], du0, du1;
  unpack_seg(seg_z, img, du0, du1);
  const D4 xj = P.cpos[k];
  const double q[3] = {xq.x, xq.y, xq.z};
  const double p[3] = {xj.x, xj.y, xj.z};
  const int D = 3 - fg.eoff;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if (e < fg.eoff) continue;
    const double cur = __dadd_rn(q[e], __dmul_rn((double)img[e], fg.L[e]));
    P.dx_out[slot * D + (e - fg.eoff)] = __dsub_rn(p[e], cur);
  }
}

// Per-warp shared state: the segment list of one batch of rows, its length
// prefix, and one staged tile of candidates.
struct WarpSeg {
  int4 seg[SEG_CAP];      // start, end, packed(img, du0, du1), c2shift
  float4 segf[SEG_CAP];   // du0, du1, c2shift as exact floats (staging offsets)
  int off[SEG_CAP + 1];   // exclusive prefix of segment lengths
};

// Build the candidate segments of rows [row0, row0+32) of the unit's stencil
// into ws.seg (warp-cooperative: one row per lane, up to three image splits
// along e2).  Returns the number of segments; ws.off holds the length prefix.
__device__ __forceinline__ int build_segments(const KParams &P, const int lo[3], const int hi[3],
                                              int a0, int a1, int R1, int nrows, int row0,
                                              WarpSeg &ws, int lane) {
  const FineGrid &fg = P.fg;
  int4 mine[3];
  bool has[3] = {false, false, false};
  const int t = row0 + lane;
  int u0s = 0, u1s = 0;
  if (t < nrows) {
    const int u0 = a0 + t / R1, u1 = a1 + t % R1;
    u0s = u0;
    u1s = u1;
    const int g0c = max(max(lo[0] - u0, u0 - hi[0]) - 1, 0);
    const int g1c = max(max(lo[1] - u1, u1 - hi[1]) - 1, 0);
    int ext;
    if (P.lnorm == -1) {
      // the chebyshev ball is the whole stencil box: no euclidean pruning
      ext = fg.K[2];
    } else if (g0c < EXT_TAB && g1c < EXT_TAB) {
      // euclidean pruning also serves the manhattan ball, which lies inside
      ext = P.ext[g0c * EXT_TAB + g1c];
    } else {
      const double g0 = g0c * fg.h[0], g1 = g1c * fg.h[1];
      const double rem = P.prune2 - g0 * g0 - g1 * g1;
      ext = rem < 0.0 ? -1 : min((int)floor(sqrt(rem) / fg.h[2]), fg.K[2]);
    }
    if (ext >= 0) {
      int w0 = u0, i0 = 0, w1 = u1, i1 = 0;
      if (u0 < 0) { w0 = u0 + fg.m[0]; i0 = 1; } else if (u0 >= fg.m[0]) { w0 = u0 - fg.m[0]; i0 = -1; }
      if (u1 < 0) { w1 = u1 + fg.m[1]; i1 = 1; } else if (u1 >= fg.m[1]) { w1 = u1 - fg.m[1]; i1 = -1; }
      const int a2 = max(lo[2] - 1 - ext, lo[2] - fg.K[2]);
      const int b2 = min(hi[2] + 1 + ext, hi[2] + fg.K[2]);
      const uint32_t rowbase = ((uint32_t)w0 * fg.m[1] + w1) * (uint32_t)fg.m[2];
      const int m2 = fg.m[2];
#pragma unroll
      for (int sgi = 0; sgi < 3; ++sgi) {
        if (sgi != 1 && !fg.periodic[2]) continue;
        const int slo = sgi == 0 ? -m2 : (sgi == 1 ? 0 : m2);
        const int shi = sgi == 0 ? -1 : (sgi == 1 ? m2 - 1 : 2 * m2 - 1);
        const int sa = max(a2, slo), sb = min(b2, shi);
        if (sa > sb) continue;
        const int i2 = 1 - sgi;            // image +1, 0, -1
        const int shift = i2 * m2;         // wrapped w2 = u2 + shift
        const uint32_t start = P.cell_start[rowbase + (uint32_t)(sa + shift)];
        const uint32_t end = P.cell_start[rowbase + (uint32_t)(sb + shift) + 1];
        if (start >= end) continue;
        const int z = (i0 + 1) | ((i1 + 1) << 2) | ((i2 + 1) << 4) |
                      ((u0 - lo[0] + 2048) << 6) | ((u1 - lo[1] + 2048) << 18);
        mine[sgi] = make_int4((int)start, (int)end, z, -shift - lo[2]);
        has[sgi] = true;
      }
    }
  }
  // compact into the shared list
  const unsigned lt = (1u << lane) - 1u;
  int base = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const unsigned m = __ballot_sync(0xffffffffu, has[k]);
    if (has[k]) {
      const int slot = base + __popc(m & lt);
      ws.seg[slot] = mine[k];
      ws.segf[slot] = make_float4((float)(u0s - lo[0]), (float)(u1s - lo[1]), (float)mine[k].w, 0.f);
    }
    base += __popc(m);
  }
  __syncwarp();
  // exclusive prefix of the lengths: lane l owns entries 3l..3l+2
  int len[3], s = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int i = 3 * lane + k;
    len[k] = i < base ? ws.seg[i].y - ws.seg[i].x : 0;
    s += len[k];
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  int run = incl - s;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int i = 3 * lane + k;
    if (i < base) ws.off[i] = run;
    run += len[k];
  }
  if (lane == 31) ws.off[base] = run;  // total
  __syncwarp();
  return base;
}

// Segment holding flattened candidate t (off[s] <= t < off[s+1]).
__device__ __forceinline__ int find_seg(const WarpSeg &ws, int nseg, int t) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ws.off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

constexpr int STAGE = 64;  // candidates staged per round (two per lane)

// Internal kernel tag: Wendland C2 in a mixed-precision matvec whose kernel
// support 1/p0 is no larger than the search radius (p0 * r >= 1 - 1e-9).  The kernel
// then vanishes at and beyond the cut-off to fourth order, so the clamp
// max(1 - q, 0) is the whole cut-off test: a pair whose FP32 and FP64
// classifications differ has |q - 1| <= delta with delta ~ 1e-5 (the FP32
// rounding band of d^2 relative to r^2), and contributes at most
// 5 delta^4 |b_j| < 1e-19 |b_j| either way -- far below the FP32 term
// precision -- so no pair needs the exact FP64 re-test.  Coordinates are
// staged pre-scaled by p0, making d^2 = q^2 directly.
constexpr int K_WEND_CUT = 100 + ABX_K_WENDLAND_C2;

struct WarpTile32 {
  float4 p[STAGE];
  // the same candidates as pairs for the packed FP32x2 loop:
  // pp[2h] = (x_a, x_b, y_a, y_b), pp[2h+1] = (z_a, z_b, b_a, b_b), a = 2h, b = 2h+1
  float4 pp[STAGE + 2];
  int2 meta[STAGE];  // column kernel index, segment index
};

// Hardware reciprocal square root (MUFU, ~2 ulp), flush-to-zero: callers
// keep x >= 1e-30 so that no denormal or zero reaches it.
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Wendland C2 of two pairs with the cut-off folded into the clamp
// t = max(1 - q, 0): exactly zero for q >= 1.
__device__ __forceinline__ float2 kern32x2_wendland_clamped(float2 dd, const KParams &P) {
  const float2 r = make_float2(sqrt_approx(dd.x), sqrt_approx(dd.y));
  const float2 q = __fmul2_rn(r, make_float2(P.p0f, P.p0f));
  float2 t = __ffma2_rn(q, make_float2(-1.f, -1.f), make_float2(1.f, 1.f));
  t.x = fmaxf(t.x, 0.f);
  t.y = fmaxf(t.y, 0.f);
  const float2 t2 = __fmul2_rn(t, t);
  const float2 t4 = __fmul2_rn(t2, t2);
  const float2 pw = __ffma2_rn(q, make_float2(4.f, 4.f), make_float2(1.f, 1.f));
  return __fmul2_rn(t4, pw);
}

// Kernel values of two pairs at once on the packed FP32x2 pipe.
template <int KIND> __device__ __forceinline__ float2 kern32x2(float2 dd, const KParams &P) {
  if (KIND == ABX_K_CONST) return make_float2(P.p0f, P.p0f);
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) {
    const float2 e = __fmul2_rn(dd, make_float2(P.c_exp2, P.c_exp2));
    return make_float2(ex2_approx(e.x), ex2_approx(e.y));
  }
  const float2 r = make_float2(sqrt_approx(dd.x), sqrt_approx(dd.y));
  if (KIND == ABX_K_WENDLAND_C2) {
    const float2 q = __fmul2_rn(r, make_float2(P.p0f, P.p0f));
    const float2 t = __ffma2_rn(q, make_float2(-1.f, -1.f), make_float2(1.f, 1.f));
    const float2 t2 = __fmul2_rn(t, t);
    const float2 t4 = __fmul2_rn(t2, t2);
    const float2 pw = __ffma2_rn(q, make_float2(4.f, 4.f), make_float2(1.f, 1.f));
    return __fmul2_rn(t4, pw);
  }
  if (KIND == ABX_K_LAPLACE) {
    const float2 a = __fadd2_rn(r, make_float2(P.p0f, P.p0f));
    return make_float2(__fdividef(1.f, a.x), __fdividef(1.f, a.y));
  }
  if (KIND == ABX_K_MULTIQUADRIC) {
    const float2 a = __fadd2_rn(dd, make_float2(P.p0f, P.p0f));
    return make_float2(sqrt_approx(a.x), sqrt_approx(a.y));
  }
  return make_float2(0.f, 0.f);
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Unit prologue shared by both kernels: the warp's anchor-cell box [lo, hi]
// and the row range of its stencil.
__device__ __forceinline__ void unit_box(const KParams &P, const int4 qc, bool active, int lo[3],
                                         int hi[3], int &a0, int &a1, int &R1, int &nrows) {
  const FineGrid &fg = P.fg;
  lo[0] = hi[0] = qc.x;
  lo[1] = hi[1] = qc.y;
  lo[2] = hi[2] = qc.z;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int a = active ? lo[e] : 0x7fffffff, b = active ? hi[e] : -0x7fffffff;
    lo[e] = __reduce_min_sync(0xffffffffu, a);
    hi[e] = __reduce_max_sync(0xffffffffu, b);
  }
  a0 = max(lo[0] - fg.K[0], fg.periodic[0] ? -fg.m[0] : 0);
  const int b0 = min(hi[0] + fg.K[0], fg.periodic[0] ? 2 * fg.m[0] - 1 : fg.m[0] - 1);
  a1 = max(lo[1] - fg.K[1], fg.periodic[1] ? -fg.m[1] : 0);
  const int b1 = min(hi[1] + fg.K[1], fg.periodic[1] ? 2 * fg.m[1] - 1 : fg.m[1] - 1);
  R1 = b1 - a1 + 1;
  const int R0 = b0 - a0 + 1;
  nrows = (R0 > 0 && R1 > 0) ? R0 * R1 : 0;
}

// Mixed-precision pair kernel.  Per unit (one warp, <= 32 queries):
//   rows of the stencil -> segment list -> flattened candidate stream, 32 at a
//   time -> each lane stages one candidate (FP32 offset from the unit's
//   reference corner) and keeps it only if it lies within r of the warp's
//   query bounding box -> every lane tests its query against the kept
//   candidates.  Pairs with d2 <= r2lo are accepted in the branch-free loop;
//   pairs in the rounding band (r2lo, r2hi] are re-decided afterwards with the
//   exact FP64 test, which is rare enough to run divergently.
// FP32 distance of a staged pair in the search norm (2: squared euclidean,
// 1: manhattan, -1: chebyshev), compared against the FP32 thresholds.
template <int NORM> __device__ __forceinline__ float norm32(float d0, float d1, float d2) {
  if (NORM == 1) return fabsf(d0) + fabsf(d1) + fabsf(d2);
  if (NORM == -1) return fmaxf(fabsf(d0), fmaxf(fabsf(d1), fabsf(d2)));
  return fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
}

template <int POL, int KIND, int NORM = 2>
__global__ void __launch_bounds__(WARPS_PER_CTA * 32, 7)
    k_pairs_mixed(KParams P) {
  static_assert(NORM == 2 || POL != POL_MATVEC, "matvecs use the euclidean distance");
  __shared__ WarpSeg seg_all[WARPS_PER_CTA];
  __shared__ WarpTile32 tile_all[WARPS_PER_CTA];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  WarpSeg &ws = seg_all[wid];
  WarpTile32 &sm = tile_all[wid];
  const FineGrid &fg = P.fg;
  const unsigned lt = (1u << lane) - 1u;
  constexpr bool WCUT = KIND == K_WEND_CUT;
  const float sc = WCUT ? P.p0f : 1.f;  // staging scale (d^2 = q^2 for WCUT)
  for (;;) {
    int unit = 0;
    if (lane == 0) unit = atomicAdd(P.counter, 1);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    if (unit >= P.nunits) break;
    const int2 U = P.units[unit];
    const bool active = lane < U.y;
    const int qi = U.x + (active ? lane : 0);
    const int4 qc = P.qcell[qi];
    const float4 ql = P.qloc[qi];
    int lo[3], hi[3], a0, a1, R1, nrows;
    unit_box(P, qc, active, lo, hi, a0, a1, R1, nrows);
    const float pq0 = fmaf((float)(qc.x - lo[0]), fg.hf[0], ql.x);
    const float pq1 = fmaf((float)(qc.y - lo[1]), fg.hf[1], ql.y);
    const float pq2 = fmaf((float)(qc.z - lo[2]), fg.hf[2], ql.z);
    // warp bounding box of the query offsets (inactive lanes repeat lane 0)
    const float bl0 = warp_min(pq0), bh0 = warp_max(pq0);
    const float bl1 = warp_min(pq1), bh1 = warp_max(pq1);
    const float bl2 = warp_min(pq2), bh2 = warp_max(pq2);
    // the box as centre and half-width, the half-width rounded outwards (a
    // wider box only keeps more candidates; none within r is dropped)
    const float bc0 = 0.5f * (bl0 + bh0), bw0 = __fadd_ru(0.5f * (bh0 - bl0), 1e-6f * (fabsf(bl0) + fabsf(bh0)));
    const float bc1 = 0.5f * (bl1 + bh1), bw1 = __fadd_ru(0.5f * (bh1 - bl1), 1e-6f * (fabsf(bl1) + fabsf(bh1)));
    const float bc2 = 0.5f * (bl2 + bh2), bw2 = __fadd_ru(0.5f * (bh2 - bl2), 1e-6f * (fabsf(bl2) + fabsf(bh2)));
    // rounding band: every staged coordinate lies within `span` cells of the
    // reference corner, so an FP32 offset carries < (3*span+2)*h*2^-24 error
    // and a difference of two < edx = (span+2)*h*2^-20; |d2_f32 - d2| <= band.
    int span = 0;
#pragma unroll
    for (int e = 0; e < 3; ++e) span = max(span, hi[e] - lo[e] + 2 * fg.K[e] + 2);
    const double hmax = fmax(fmax(fg.h[0] * (fg.eoff <= 0), fg.h[1] * (fg.eoff <= 1)), fg.h[2]);
    const double edx = (double)(span + 2) * hmax * 9.5367431640625e-07;
    const double band = 2.0 * 1.7320508075688772 * (P.r + edx) * edx + 3.0 * edx * edx +
                        4.0 * 5.960464477539063e-08 * P.r2 + 1e-300;
    // manhattan / chebyshev: each FP32 |d_e| is within edx of the exact one,
    // the sum of three adds <= 2 roundings of a value below 3 r
    const double nband = NORM == 1 ? 3.0 * edx + 6.0 * 5.960464477539063e-08 * 3.0 * P.r + 1e-300
                                   : edx + 2.0 * 5.960464477539063e-08 * P.r + 1e-300;
    // (when the band reaches below 0 nothing is accepted outright: two
    // distinct points may share an FP32 offset, d = 0, yet lie outside a
    // radius smaller than the band)
    const double lo_thr = NORM == 2 ? P.r2 - band : P.thr - nband;
    const float r2lo = lo_thr > 0.0 ? __double2float_rd(lo_thr) : -1.0f;
    const float r2hi = NORM == 2 ? __double2float_ru(P.r2 + band) : __double2float_ru(P.thr + nband);
    // box test: euclidean for norms 2 and 1 (the manhattan ball lies inside
    // the euclidean one), a max-norm test for the chebyshev ball
    const float r2box = __double2float_ru((P.r2 + band) * (1.0 + 1e-6) + 1e-300);
    const float rbox_inf = __double2float_ru((P.thr + nband) * (1.0 + 1e-6) + 1e-300);
    // band as |d2 - r2mid| <= r2half, widened by a few ulps so that the FP32
    // subtraction never shrinks it below (r2lo, r2hi]
    const float r2mid = (float)(0.5 * ((double)r2lo + (double)r2hi));
    const float r2half =
        __double2float_ru(0.5 * ((double)r2hi - (double)r2lo) + 8.0 * 5.960464477539063e-08 * P.r2);
    D4 xq;
    bool have_xq = false;
    double acc64 = 0.0;
    int count = 0;
    int64_t out_off = 0;
    if (POL == POL_LIST && active) out_off = P.rowptr[qi];
    if (POL == POL_LIST && P.dx_out) {
      xq = P.qpos[qi];
      have_xq = true;
    }

    for (int row0 = 0; row0 < nrows; row0 += 32) {
      const int nseg = build_segments(P, lo, hi, a0, a1, R1, nrows, row0, ws, lane);
      if (nseg == 0) continue;
      const int total = ws.off[nseg];
      int cur = 0;  // this lane's segment; its candidate index only grows
      for (int t0 = 0; t0 < total; t0 += STAGE) {
        int nt = 0;
        // staging in three phases so that the global loads of every
        // sub-round are in flight together: (1) candidate indices from the
        // segment list, (2) positions and weights, (3) bounding-box test and
        // compaction into shared memory
        constexpr int NS = STAGE / 32;
        int kk[NS], sx[NS];
        float4 so[NS];
#pragma unroll
        for (int sub = 0; sub < NS; ++sub) {
          const int t = t0 + sub * 32 + lane;
          kk[sub] = -1;
          sx[sub] = 0;
          so[sub] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (t < total) {
            while (cur + 1 < nseg && ws.off[cur + 1] <= t) ++cur;
            sx[sub] = cur;
            kk[sub] = ws.seg[cur].x + (t - ws.off[cur]);
            so[sub] = ws.segf[cur];
          }
        }
        float4 cls[NS];
        float bws[NS];
#pragma unroll
        for (int sub = 0; sub < NS; ++sub) {
          cls[sub] = make_float4(0.f, 0.f, 0.f, 0.f);
          bws[sub] = 0.f;
          if (kk[sub] >= 0) {
            cls[sub] = __ldg(&P.cloc[kk[sub]]);
            if (POL == POL_MATVEC) bws[sub] = __ldg(&P.b32[kk[sub]]);
          }
        }
#pragma unroll
        for (int sub = 0; sub < NS; ++sub) {
          bool keep = false;
          float4 st;
          const int k = kk[sub], sidx = sx[sub];
          if (k >= 0) {
            const float4 cl = cls[sub];
            // offsets from the unit's reference corner: whole cells (exact
            // small integers) times the cell size plus the in-cell offset
            st.x = fmaf(so[sub].x, fg.hf[0], cl.x);
            st.y = fmaf(so[sub].y, fg.hf[1], cl.y);
            st.z = fmaf(cl.w + so[sub].z, fg.hf[2], cl.z);
            const float e0 = fmaxf(fabsf(st.x - bc0) - bw0, 0.f);
            const float e1 = fmaxf(fabsf(st.y - bc1) - bw1, 0.f);
            const float e2 = fmaxf(fabsf(st.z - bc2) - bw2, 0.f);
            keep = NORM == -1 ? fmaxf(e0, fmaxf(e1, e2)) <= rbox_inf
                              : fmaf(e2, e2, fmaf(e1, e1, e0 * e0)) <= r2box;
            st.w = bws[sub];
          }
          const unsigned km = __ballot_sync(0xffffffffu, keep);
          if (WCUT) {
            // natural order, one 16-byte store per lane (no bank conflicts);
            // repacked into candidate pairs below
            if (keep) sm.p[nt + __popc(km & lt)] = make_float4(st.x * sc, st.y * sc, st.z * sc, st.w);
          } else if (keep) {
            const int slot = nt + __popc(km & lt);
            sm.p[slot] = st;
            sm.meta[slot] = make_int2(k, sidx);
            if (POL == POL_MATVEC) {
              float *pf = reinterpret_cast<float *>(&sm.pp[2 * (slot >> 1)]);
              const int o = slot & 1;
              pf[o] = st.x;
              pf[2 + o] = st.y;
              pf[4 + o] = st.z;
              pf[6 + o] = st.w;
            }
          }
          nt += __popc(km);
        }
        __syncwarp();
        if (WCUT) {
          // pairs for the packed loop; an odd tail is paired with a far-away
          // candidate of weight 0 (the clamp zeroes it)
          for (int h = lane; 2 * h < nt; h += 32) {
            const float4 c0 = sm.p[2 * h];
            const float4 c1 = 2 * h + 1 < nt ? sm.p[2 * h + 1] : make_float4(1e4f, 1e4f, 1e4f, 0.f);
            sm.pp[2 * h] = make_float4(c0.x, c1.x, c0.y, c1.y);
            sm.pp[2 * h + 1] = make_float4(c0.z, c1.z, c0.w, c1.w);
          }
        }
        if (!WCUT && POL == POL_MATVEC && lane == 0 && (nt & 1)) {
          // pad an odd tile with a far-away candidate of weight 0 (finite, so
          // that every kernel formula stays finite and the clamp/select zeroes it)
          float *pf = reinterpret_cast<float *>(&sm.pp[2 * (nt >> 1)]);
          pf[1] = pf[3] = pf[5] = 1e4f;
          pf[7] = 0.f;
        }
        __syncwarp();
        float acc32 = 0.f;
        bool need = false;
        if (WCUT) {
          // one query against two candidates per packed FP32x2 instruction;
          // coordinates in units of the kernel support, so q = |dx|
          const float2 nqx = make_float2(-pq0 * sc, -pq0 * sc), nqy = make_float2(-pq1 * sc, -pq1 * sc),
                       nqz = make_float2(-pq2 * sc, -pq2 * sc);
          float2 acc2 = make_float2(0.f, 0.f);
          const int npair = (nt + 1) >> 1;
#pragma unroll 8
          for (int h = 0; h < npair; ++h) {
            const float4 A = sm.pp[2 * h], B = sm.pp[2 * h + 1];
            const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nqx);
            const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nqy);
            const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nqz);
            // d^2 (+1e-30, so that rsqrt stays finite for the self pair)
            float2 dd = __ffma2_rn(dx, dx, make_float2(1e-30f, 1e-30f));
            dd = __ffma2_rn(dy, dy, dd);
            dd = __ffma2_rn(dz, dz, dd);
            const float2 rs = make_float2(rsqrt_approx(dd.x), rsqrt_approx(dd.y));
            // t = max(1 - q, 0), q = d^2 / d, as saturating FMAs (q >= 0, so
            // [0,1] is the clamp); then 4q + 1 = 5 - 4t wherever t > 0
            const float2 t = make_float2(__saturatef(fmaf(-dd.x, rs.x, 1.f)),
                                         __saturatef(fmaf(-dd.y, rs.y, 1.f)));
            const float2 t2 = __fmul2_rn(t, t);
            const float2 pw = __ffma2_rn(t, make_float2(-4.f, -4.f), make_float2(5.f, 5.f));
            const float2 t4 = __fmul2_rn(t2, t2);
            acc2 = __ffma2_rn(__fmul2_rn(t4, pw), make_float2(B.z, B.w), acc2);
          }
          acc32 = acc2.x + acc2.y;
        } else if (POL == POL_MATVEC) {
          // one query against two candidates per packed FP32x2 instruction
          const float2 nqx = make_float2(-pq0, -pq0), nqy = make_float2(-pq1, -pq1),
                       nqz = make_float2(-pq2, -pq2);
          float2 acc2 = make_float2(0.f, 0.f);
          const int npair = (nt + 1) >> 1;
#pragma unroll 2
          for (int h = 0; h < npair; ++h) {
            const float4 A = sm.pp[2 * h], B = sm.pp[2 * h + 1];
            const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nqx);
            const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nqy);
            const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nqz);
            float2 dd = __fmul2_rn(dx, dx);
            dd = __ffma2_rn(dy, dy, dd);
            dd = __ffma2_rn(dz, dz, dd);
            float2 w;
            if (KIND == ABX_K_WENDLAND_C2) {
              // the kernel vanishes for q >= 1: the clamp is the cut-off for
              // every pair outside the rounding band (d2 > r2hi means q > 1),
              // and band pairs are flagged for the exact test below
              const float2 bd = __fadd2_rn(dd, make_float2(-r2mid, -r2mid));
              need |= (fabsf(bd.x) <= r2half) | (fabsf(bd.y) <= r2half);
              w = kern32x2_wendland_clamped(dd, P);
            } else {
              const bool ia = dd.x <= r2lo, ib = dd.y <= r2lo;
              need |= ((dd.x > r2lo) & (dd.x <= r2hi)) | ((dd.y > r2lo) & (dd.y <= r2hi));
              w = kern32x2<KIND>(dd, P);
              w.x = ia ? w.x : 0.f;
              w.y = ib ? w.y : 0.f;
            }
            acc2 = __ffma2_rn(w, make_float2(B.z, B.w), acc2);
          }
          acc32 = acc2.x + acc2.y;
        }
#pragma unroll 4
        for (int j = 0; j < nt && POL != POL_MATVEC; ++j) {
          const float4 c = sm.p[j];
          const float dd = norm32<NORM>(c.x - pq0, c.y - pq1, c.z - pq2);
          const bool in = dd <= r2lo;
          need |= (dd > r2lo) & (dd <= r2hi);
          if (POL == POL_MATVEC) {
            const float w = kern32<KIND>(dd, P);
            acc32 = fmaf(in ? w : 0.f, c.w, acc32);
          }
          if (POL == POL_COUNT) count += in ? 1 : 0;
          if (POL == POL_LIST && in && active) {
            const int2 mt = sm.meta[j];
            if (P.dx_out) write_dx(P, out_off, xq, mt.x, ws.seg[mt.y].z);
            P.cols_out[out_off++] = (int32_t)P.cperm[mt.x];
          }
        }
        if (!WCUT && __any_sync(0xffffffffu, need)) {
          // rare: decide the band pairs with the reference's FP64 test
          if (need) {
            if (!have_xq) {
              xq = P.qpos[qi];
              have_xq = true;
            }
            for (int j = 0; j < nt; ++j) {
              const float4 c = sm.p[j];
              const float dd = norm32<NORM>(c.x - pq0, c.y - pq1, c.z - pq2);
              const bool wend = POL == POL_MATVEC && KIND == ABX_K_WENDLAND_C2;
              const bool flagged = wend ? fabsf(__fadd_rn(dd, -r2mid)) <= r2half
                                        : (dd > r2lo && dd <= r2hi);
              if (flagged) {
                const int2 mt = sm.meta[j];
                int img[3], du0, du1;
                unpack_seg(ws.seg[mt.y].z, img, du0, du1);
                const bool inside = !(exact_norm(xq, P.cpos[mt.x], img, fg, NORM) > P.thr);
                if (wend) {
                  // the packed loop added the clamped value: take it back out
                  // for pairs the FP64 test rejects
                  if (!inside) acc32 -= kern32x2_wendland_clamped(make_float2(dd, dd), P).x * c.w;
                } else if (inside) {
                  if (POL == POL_MATVEC) acc32 = fmaf(kern32<KIND>(dd, P), c.w, acc32);
                  if (POL == POL_COUNT) ++count;
                  if (POL == POL_LIST && active) {
                    if (P.dx_out) write_dx(P, out_off, xq, mt.x, ws.seg[mt.y].z);
                    P.cols_out[out_off++] = (int32_t)P.cperm[mt.x];
                  }
                }
              }
            }
          }
          __syncwarp();
        }
        if (POL == POL_MATVEC) acc64 += (double)acc32;
        __syncwarp();
      }
    }
    if (active) {
      if (POL == POL_MATVEC) P.c[qi] = acc64;
      if (POL == POL_COUNT) P.counts[qi] = count;
    }
  }
}

// Per-warp staging of the FP64 matvec: the candidates kept by the warp's
// bounding-box test, as FP32 offsets (for the prefilter) and as FP64
// positions shifted by their periodic image (x_j - image*L, for the kernel
// value), with their weights and (column index, segment) for the exact test.
struct WarpTile64 {
  float4 pf[STAGE];
  double ux[STAGE], uy[STAGE], uz[STAGE], b[STAGE], s[STAGE];
  int2 meta[STAGE];
};

// FP64 sparse matvec: the reference's arithmetic for every accepted pair,
// FP64 work only for accepted pairs.  Per staged tile of <= 64 candidates:
//  (1) every lane classifies all candidates with the FP32 offsets into
//      accepted (d2 <= r2lo), rejected (d2 > r2hi) and the rounding band,
//      where the reference's exact FP64 test decides (rare); the result is a
//      64-bit mask of this lane's neighbours among the candidates;
//  (2) every lane walks its own mask and evaluates the FP64 distance, kernel
//      and product for those pairs only.
// The warp then pays FP64 issue for max over lanes of its neighbour count,
// not for every (query, candidate) combination.  The distance for the kernel
// value is |(x_j - image*L) - x_i|, which differs from the reference's
// x_j - (x_i + image*L) by at most an ulp of the box length (the acceptance
// decision itself is exact); the row sum order differs from the reference's.
template <int POL, int KIND>
__global__ void __launch_bounds__(WARPS_PER_CTA * 32, 6)
    k_pairs_fp64(KParams P) {
  __shared__ WarpSeg seg_all[WARPS_PER_CTA];
  __shared__ WarpTile64 tile_all[WARPS_PER_CTA];
  static_assert(POL == POL_MATVEC, "the FP64 pair kernel computes matvecs only");
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  WarpSeg &ws = seg_all[wid];
  WarpTile64 &sm = tile_all[wid];
  const FineGrid &fg = P.fg;
  const unsigned lt = (1u << lane) - 1u;
  for (;;) {
    int unit = 0;
    if (lane == 0) unit = atomicAdd(P.counter, 1);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    if (unit >= P.nunits) break;
    const int2 U = P.units[unit];
    const bool active = lane < U.y;
    const int qi = U.x + (active ? lane : 0);
    const int4 qc = P.qcell[qi];
    const float4 ql = P.qloc[qi];
    int lo[3], hi[3], a0, a1, R1, nrows;
    unit_box(P, qc, active, lo, hi, a0, a1, R1, nrows);
    const float pq0 = fmaf((float)(qc.x - lo[0]), fg.hf[0], ql.x);
    const float pq1 = fmaf((float)(qc.y - lo[1]), fg.hf[1], ql.y);
    const float pq2 = fmaf((float)(qc.z - lo[2]), fg.hf[2], ql.z);
    const float bl0 = warp_min(pq0), bh0 = warp_max(pq0);
    const float bl1 = warp_min(pq1), bh1 = warp_max(pq1);
    const float bl2 = warp_min(pq2), bh2 = warp_max(pq2);
    const float bc0 = 0.5f * (bl0 + bh0), bw0 = __fadd_ru(0.5f * (bh0 - bl0), 1e-6f * (fabsf(bl0) + fabsf(bh0)));
    const float bc1 = 0.5f * (bl1 + bh1), bw1 = __fadd_ru(0.5f * (bh1 - bl1), 1e-6f * (fabsf(bl1) + fabsf(bh1)));
    const float bc2 = 0.5f * (bl2 + bh2), bw2 = __fadd_ru(0.5f * (bh2 - bl2), 1e-6f * (fabsf(bl2) + fabsf(bh2)));
    // rounding band of the FP32 d2 (the same bound as the mixed kernel's)
    int span = 0;
#pragma unroll
    for (int e = 0; e < 3; ++e) span = max(span, hi[e] - lo[e] + 2 * fg.K[e] + 2);
    const double hmax = fmax(fmax(fg.h[0] * (fg.eoff <= 0), fg.h[1] * (fg.eoff <= 1)), fg.h[2]);
    const double edx = (double)(span + 2) * hmax * 9.5367431640625e-07;
    const double band = 2.0 * 1.7320508075688772 * (P.r + edx) * edx + 3.0 * edx * edx +
                        4.0 * 5.960464477539063e-08 * P.r2 + 1e-300;
    const float r2lo = P.r2 - band > 0.0 ? __double2float_rd(P.r2 - band) : -1.0f;
    const float r2hi = __double2float_ru(P.r2 + band);
    const float r2box = __double2float_ru((P.r2 + band) * (1.0 + 1e-6) + 1e-300);
    const D4 xq = P.qpos[qi];
    const double si = (KIND == ABX_K_SCALAR_SUM) ? P.s_row[qi] : 0.0;
    double acc = 0.0;

    for (int row0 = 0; row0 < nrows; row0 += 32) {
      const int nseg = build_segments(P, lo, hi, a0, a1, R1, nrows, row0, ws, lane);
      if (nseg == 0) continue;
      const int total = ws.off[nseg];
      int cur = 0;
      for (int t0 = 0; t0 < total; t0 += STAGE) {
        constexpr int NS = STAGE / 32;
        int kk[NS], sx[NS];
        float4 so[NS];
#pragma unroll
        for (int sub = 0; sub < NS; ++sub) {
          const int t = t0 + sub * 32 + lane;
          kk[sub] = -1;
          sx[sub] = 0;
          so[sub] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (t < total) {
            while (cur + 1 < nseg && ws.off[cur + 1] <= t) ++cur;
            sx[sub] = cur;
            kk[sub] = ws.seg[cur].x + (t - ws.off[cur]);
            so[sub] = ws.segf[cur];
          }
        }
        float4 cls[NS];
#pragma unroll
        for (int sub = 0; sub < NS; ++sub)
          cls[sub] = kk[sub] >= 0 ? __ldg(&P.cloc[kk[sub]]) : make_float4(0.f, 0.f, 0.f, 0.f);
        int nt = 0;
#pragma unroll
        for (int sub = 0; sub < NS; ++sub) {
          bool keep = false;
          float4 st = make_float4(0.f, 0.f, 0.f, 0.f);
          const int k = kk[sub];
          if (k >= 0) {
            const float4 cl = cls[sub];
            st.x = fmaf(so[sub].x, fg.hf[0], cl.x);
            st.y = fmaf(so[sub].y, fg.hf[1], cl.y);
            st.z = fmaf(cl.w + so[sub].z, fg.hf[2], cl.z);
            const float e0 = fmaxf(fabsf(st.x - bc0) - bw0, 0.f);
            const float e1 = fmaxf(fabsf(st.y - bc1) - bw1, 0.f);
            const float e2 = fmaxf(fabsf(st.z - bc2) - bw2, 0.f);
            keep = fmaf(e2, e2, fmaf(e1, e1, e0 * e0)) <= r2box;
          }
          const unsigned km = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            const int slot = nt + __popc(km & lt);
            int img[3], du0, du1;
            unpack_seg(ws.seg[sx[sub]].z, img, du0, du1);
            const D4 pj = P.cpos[k];
            sm.pf[slot] = st;
            sm.ux[slot] = __dsub_rn(pj.x, (double)img[0] * fg.L[0]);
            sm.uy[slot] = __dsub_rn(pj.y, (double)img[1] * fg.L[1]);
            sm.uz[slot] = __dsub_rn(pj.z, (double)img[2] * fg.L[2]);
            sm.b[slot] = P.b64[k];
            if (KIND == ABX_K_SCALAR_SUM) sm.s[slot] = P.s_col[k];
            sm.meta[slot] = make_int2(k, sx[sub]);
          }
          nt += __popc(km);
        }
        __syncwarp();
        // (1) this lane's neighbours among the nt staged candidates
        unsigned m0 = 0u, m1 = 0u, band0 = 0u, band1 = 0u;
        if (active) {
          for (int j = 0; j < nt; ++j) {
            const float4 c = sm.pf[j];
            const float d0 = c.x - pq0, d1 = c.y - pq1, d2v = c.z - pq2;
            const float dd = fmaf(d2v, d2v, fmaf(d1, d1, d0 * d0));
            const unsigned in = dd <= r2lo ? 1u : 0u;
            const unsigned bd = (dd > r2lo && dd <= r2hi) ? 1u : 0u;
            if (j < 32) {
              m0 |= in << j;
              band0 |= bd << j;
            } else {
              m1 |= in << (j - 32);
              band1 |= bd << (j - 32);
            }
          }
        }
        // rare: the reference's exact FP64 test for pairs in the band
        while (band0 | band1) {
          const int j = band0 ? __ffs(band0) - 1 : 32 + __ffs(band1) - 1;
          if (j < 32) band0 &= band0 - 1u; else band1 &= band1 - 1u;
          const int2 mt = sm.meta[j];
          int img[3], du0, du1;
          unpack_seg(ws.seg[mt.y].z, img, du0, du1);
          if (!(exact_d2(xq, P.cpos[mt.x], img, fg) > P.r2)) {
            if (j < 32) m0 |= 1u << j; else m1 |= 1u << (j - 32);
          }
        }
        // (2) FP64 distance, kernel and product for this lane's neighbours
        while (m0 | m1) {
          const int j = m0 ? __ffs(m0) - 1 : 32 + __ffs(m1) - 1;
          if (j < 32) m0 &= m0 - 1u; else m1 &= m1 - 1u;
          const double dx = sm.ux[j] - xq.x, dy = sm.uy[j] - xq.y, dz = sm.uz[j] - xq.z;
          const double d2 = fma(dz, dz, fma(dy, dy, dx * dx));
          acc = fma(kern64<KIND>(d2, P, si, sm.s[j]), sm.b[j], acc);
        }
        __syncwarp();
      }
    }
    if (active) P.c[qi] = acc;
  }
}

__global__ void k_gather_b(const double *__restrict__ b, const uint32_t *__restrict__ perm,
                           int64_t n, float *__restrict__ b32, double *__restrict__ b64) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double v = b[perm[k]];
  if (b32) b32[k] = (float)v;
  if (b64) b64[k] = v;
}

__global__ void k_scatter_c(const double *__restrict__ ck, const uint32_t *__restrict__ perm,
                            int64_t n, double *__restrict__ c) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  c[perm[k]] = ck[k];
}

template <class T>
__global__ void k_scatter(const T *__restrict__ src, const uint32_t *__restrict__ perm, int64_t n,
                          T *__restrict__ dst) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  dst[perm[k]] = src[k];
}

// Largest e2 gap (in cells) that keeps a cell within the pruning distance,
// for every pair of e0/e1 gaps below EXT_TAB cells (-1: pruned).
int build_ext_table(PairLayout &L, double prune2) {
  std::vector<int> tab(EXT_TAB * EXT_TAB);
  const FineGrid &fg = L.fg;
  for (int a = 0; a < EXT_TAB; ++a)
    for (int b = 0; b < EXT_TAB; ++b) {
      const double g0 = a * fg.h[0], g1 = b * fg.h[1];
      const double rem = prune2 - g0 * g0 - g1 * g1;
      tab[a * EXT_TAB + b] =
          rem < 0.0 ? -1 : std::min((int)std::floor(std::sqrt(rem) / fg.h[2]), fg.K[2]);
    }
  ABX_TRY(L.ext.reserve(tab.size()));
  ABX_CHECK_CUDA(cudaMemcpy(L.ext.ptr, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice));
  return ABX_OK;
}

double prune_distance2(const PairLayout &L) {
  double hmax = 0;
  for (int e = 0; e < 3; ++e)
    if (e >= L.fg.eoff) hmax = std::max(hmax, L.fg.h[e]);
  const double margin = L.r * 1e-9 + hmax * 1e-9;
  return (L.r + margin) * (L.r + margin);
}

KParams base_params(const PairLayout &L) {
  KParams P{};
  P.ext = L.ext.ptr;
  P.fg = L.fg;
  P.r = L.r;
  P.r2 = L.r * L.r;
  P.lnorm = 2;
  P.thr = P.r2;
  P.prune2 = prune_distance2(L);
  P.cloc = L.cols.loc.ptr;
  P.cpos = L.cols.posk.ptr;
  P.cell_start = L.cell_start.ptr;
  P.cperm = L.cols.perm.ptr;
  P.qcell = L.rows->cell.ptr;
  P.qloc = L.rows->loc.ptr;
  P.qpos = L.rows->posk.ptr;
  P.units = L.units.ptr;
  P.nunits = L.nunits;
  P.counter = L.counter.ptr;
  return P;
}

int grid_blocks(abx_context *ctx, int nunits) {
  int blocks = ctx->num_sms * 8;
  const int need = (nunits + WARPS_PER_CTA - 1) / WARPS_PER_CTA;
  return std::max(1, std::min(blocks, need));
}

template <int POL, int KIND> int launch_pairs(abx_context *ctx, const KParams &P, bool mixed) {
  const int blocks = grid_blocks(ctx, P.nunits);
  ABX_CHECK_CUDA(cudaMemsetAsync(P.counter, 0, sizeof(int), ctx->stream));
  if (mixed) {
    k_pairs_mixed<POL, KIND><<<blocks, WARPS_PER_CTA * 32, 0, ctx->stream>>>(P);
  } else {
    if constexpr (POL == POL_MATVEC) {
      k_pairs_fp64<POL, KIND><<<blocks, WARPS_PER_CTA * 32, 0, ctx->stream>>>(P);
    } else {
      set_error("the FP64 pair kernel computes matvecs only");
      return ABX_ERR_INVALID;
    }
  }
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

// The radius search (count or list) in the norm P.lnorm.
template <int POL> int launch_search(abx_context *ctx, const KParams &P) {
  const int blocks = grid_blocks(ctx, P.nunits);
  ABX_CHECK_CUDA(cudaMemsetAsync(P.counter, 0, sizeof(int), ctx->stream));
  if (P.lnorm == 1)
    k_pairs_mixed<POL, ABX_K_CONST, 1><<<blocks, WARPS_PER_CTA * 32, 0, ctx->stream>>>(P);
  else if (P.lnorm == -1)
    k_pairs_mixed<POL, ABX_K_CONST, -1><<<blocks, WARPS_PER_CTA * 32, 0, ctx->stream>>>(P);
  else
    k_pairs_mixed<POL, ABX_K_CONST, 2><<<blocks, WARPS_PER_CTA * 32, 0, ctx->stream>>>(P);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

int launch_wend_cut(abx_context *ctx, const KParams &P) {
  const int blocks = grid_blocks(ctx, P.nunits);
  ABX_CHECK_CUDA(cudaMemsetAsync(P.counter, 0, sizeof(int), ctx->stream));
  k_pairs_mixed<POL_MATVEC, K_WEND_CUT><<<blocks, WARPS_PER_CTA * 32, 0, ctx->stream>>>(P);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

template <int POL> int launch_pairs_kind(abx_context *ctx, const KParams &P, bool mixed) {
  switch (P.kind) {
  case ABX_K_CONST: return launch_pairs<POL, ABX_K_CONST>(ctx, P, mixed);
  case ABX_K_GAUSSIAN: return launch_pairs<POL, ABX_K_GAUSSIAN>(ctx, P, mixed);
  case ABX_K_WENDLAND_C2:
    // support 1/p0 <= r up to rounding of p0 = 1/r (a support wider by a
    // relative 1e-9 adds pairs of weight <= 5e-36)
    if (POL == POL_MATVEC && mixed && P.p0 * P.r >= 1.0 - 1e-9) return launch_wend_cut(ctx, P);
    return launch_pairs<POL, ABX_K_WENDLAND_C2>(ctx, P, mixed);
  case ABX_K_COMPACT_GAUSSIAN: return launch_pairs<POL, ABX_K_COMPACT_GAUSSIAN>(ctx, P, mixed);
  case ABX_K_LAPLACE: return launch_pairs<POL, ABX_K_LAPLACE>(ctx, P, mixed);
  case ABX_K_MULTIQUADRIC: return launch_pairs<POL, ABX_K_MULTIQUADRIC>(ctx, P, mixed);
  case ABX_K_SCALAR_SUM: return launch_pairs<POL, ABX_K_SCALAR_SUM>(ctx, P, false);
  }
  set_error("unknown kernel kind %d", P.kind);
  return ABX_ERR_INVALID;
}

// Build a layout for cols (a searchable particle set) and a query set given as
// SoA FP64 (qsrc, nq, stride) -- or the column set itself when qsrc == null.
int layout_build(abx_context *ctx, abx_particles *cols, double r, const double *qsrc, int64_t nq,
                 int64_t qstride, PairLayout &L) {
  GridDesc g;
  ABX_TRY(particles_grid_desc(cols, &g));
  L.r = r;
  L.fg = make_fine_grid(g, r, std::max<int64_t>(cols->n, 1), 3);
  L.cols_version = cols->version;
  ABX_TRY(build_points(ctx, cols->pos.ptr, cols->n, cols->n, L.fg, true, L.cols));
  ABX_TRY(build_cell_start(ctx, L));
  if (!qsrc) {
    L.self = true;
    L.rows = &L.cols;
  } else {
    L.self = false;
    ABX_TRY(build_points(ctx, qsrc, nq, qstride, L.fg, false, L.rows_own));
    L.rows = &L.rows_own;
  }
  ABX_TRY(build_units(ctx, L));
  ABX_TRY(build_ext_table(L, prune_distance2(L)));
  return ABX_OK;
}

}  // namespace

int pair_layout_build(abx_operator *op) {
  abx_context *ctx = op->rows->ctx;
  if (op->pairs) delete op->pairs;
  op->pairs = new PairLayout();
  PairLayout &L = *op->pairs;
  const bool self = op->rows == op->cols;
  ABX_TRY(layout_build(ctx, op->cols, op->radius, self ? nullptr : op->rows->pos.ptr,
                       op->rows->n, op->rows->n, L));
  L.rows_version = op->rows->version;
  const int64_t nr = L.rows->n, nc = L.cols.n;
  ABX_TRY(L.bk32.reserve(nc ? nc : 1));
  ABX_TRY(L.bk64.reserve(nc ? nc : 1));
  ABX_TRY(L.ck.reserve(nr ? nr : 1));
  if (op->k.kind == ABX_K_SCALAR_SUM) {
    ABX_REQUIRE(op->rows->has_scalar && op->cols->has_scalar, ABX_ERR_STATE,
                "ABX_K_SCALAR_SUM needs a scalar column on both particle sets");
    ABX_TRY(L.sk.reserve(nc ? nc : 1));
    ABX_TRY(L.sq.reserve(nr ? nr : 1));
    if (nc)
      k_gather_b<<<ceil_div(nc, TPB), TPB, 0, ctx->stream>>>(op->cols->scalar.ptr, L.cols.perm.ptr,
                                                             nc, nullptr, L.sk.ptr);
    if (nr)
      k_gather_b<<<ceil_div(nr, TPB), TPB, 0, ctx->stream>>>(op->rows->scalar.ptr, L.rows->perm.ptr,
                                                             nr, nullptr, L.sq.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
  }
  ABX_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return ABX_OK;
}

int sparse_matvec_device(abx_operator *op, const double *b, double *c) {
  abx_context *ctx = op->rows->ctx;
  if (!op->pairs || op->pairs->cols_version != op->cols->version ||
      op->pairs->rows_version != op->rows->version)
    ABX_TRY(pair_layout_build(op));
  PairLayout &L = *op->pairs;
  const int64_t nr = L.rows->n, nc = L.cols.n;
  if (nr == 0) return ABX_OK;
  const bool mixed = op->precision == ABX_PREC_MIXED && op->k.kind != ABX_K_SCALAR_SUM;
  if (nc > 0)
    k_gather_b<<<ceil_div(nc, TPB), TPB, 0, ctx->stream>>>(
        b, L.cols.perm.ptr, nc, mixed ? L.bk32.ptr : nullptr, mixed ? nullptr : L.bk64.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  KParams P = base_params(L);
  P.kind = op->k.kind;
  P.p0 = op->k.p[0];
  P.p0f = (float)op->k.p[0];
  P.c_exp2 = (float)(-op->k.p[0] * 1.4426950408889634);
  P.b32 = L.bk32.ptr;
  P.b64 = L.bk64.ptr;
  P.s_col = L.sk.ptr;
  P.s_row = L.sq.ptr;
  P.c = L.ck.ptr;
  if (nc == 0) {
    ABX_CHECK_CUDA(cudaMemsetAsync(c, 0, nr * sizeof(double), ctx->stream));
    return ABX_OK;
  }
  ABX_TRY(launch_pairs_kind<POL_MATVEC>(ctx, P, mixed));
  k_scatter_c<<<ceil_div(nr, TPB), TPB, 0, ctx->stream>>>(L.ck.ptr, L.rows->perm.ptr, nr, c);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

namespace {
__global__ void k_aos_to_soa_q(const double *__restrict__ aos, int64_t n, int dim,
                               double *__restrict__ soa) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int d = 0; d < dim; ++d) soa[(int64_t)d * n + i] = aos[i * dim + d];
}

__global__ void k_count_to_i64(const int32_t *__restrict__ counts, const uint32_t *__restrict__ perm,
                               int64_t n, int64_t *__restrict__ rowcnt) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  rowcnt[perm[k]] = counts[k];
}

__global__ void k_rowptr_to_kernel(const int64_t *__restrict__ rowptr,
                                   const uint32_t *__restrict__ perm, int64_t n,
                                   int64_t *__restrict__ rowptr_k) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  rowptr_k[k] = rowptr[perm[k]];
}
}  // namespace

// Radius queries for arbitrary points (C ABI helpers).
int radius_query(abx_particles *p, int64_t nq, const double *q_host_or_dev, double r,
                 int32_t *counts_user, int64_t *rowptr_user, int32_t *cols_user, int64_t cap,
                 int lnorm, double *dx_user = nullptr) {
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called on this particle set");
  ABX_REQUIRE(r >= 0 && std::isfinite(r), ABX_ERR_INVALID, "invalid radius");
  ABX_REQUIRE(lnorm == 2 || lnorm == 1 || lnorm == -1, ABX_ERR_INVALID,
              "norm %d not supported (2 euclidean, 1 manhattan, -1 chebyshev)", lnorm);
  const int D = p->dim;
  const void *qd;
  ABX_TRY(p->stage_b.in(ctx, q_host_or_dev, (size_t)nq * D * sizeof(double), &qd));
  DevBuf<double> qsoa;
  ABX_TRY(qsoa.reserve((size_t)D * (nq ? nq : 1)));
  if (nq)
    k_aos_to_soa_q<<<ceil_div(nq, TPB), TPB, 0, s>>>((const double *)qd, nq, D, qsoa.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  PairLayout L;
  ABX_TRY(layout_build(ctx, p, r, qsoa.ptr, nq, nq, L));
  if (nq == 0) {
    if (rowptr_user) {
      int64_t z = 0;
      ABX_CHECK_CUDA(cudaMemcpy(rowptr_user, &z, sizeof(int64_t), cudaMemcpyDefault));
    }
    return ABX_OK;
  }
  DevBuf<int32_t> cnt_k;
  ABX_TRY(cnt_k.reserve(nq));
  KParams P = base_params(L);
  P.kind = ABX_K_CONST;
  P.lnorm = lnorm;
  P.thr = lnorm == 2 ? r * r : std::fabs(r);
  P.counts = cnt_k.ptr;
  ABX_CHECK_CUDA(cudaMemsetAsync(cnt_k.ptr, 0, nq * 4, s));
  if (p->n > 0) ABX_TRY(launch_search<POL_COUNT>(ctx, P));
  if (counts_user) {
    DevBuf<int32_t> cnt;
    ABX_TRY(cnt.reserve(nq));
    k_scatter<int32_t><<<ceil_div(nq, TPB), TPB, 0, s>>>(cnt_k.ptr, L.rows->perm.ptr, nq, cnt.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    ABX_CHECK_CUDA(cudaMemcpyAsync(counts_user, cnt.ptr, nq * 4, cudaMemcpyDefault, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  if (rowptr_user) {
    // rowptr in input order: counts -> int64 -> exclusive scan (host: nq+1)
    DevBuf<int64_t> rc;
    ABX_TRY(rc.reserve(nq));
    k_count_to_i64<<<ceil_div(nq, TPB), TPB, 0, s>>>(cnt_k.ptr, L.rows->perm.ptr, nq, rc.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    std::vector<int64_t> h(nq + 1);
    ABX_CHECK_CUDA(cudaMemcpyAsync(h.data(), rc.ptr, nq * 8, cudaMemcpyDeviceToHost, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    int64_t run = 0;
    for (int64_t i = 0; i < nq; ++i) {
      const int64_t c = h[i];
      h[i] = run;
      run += c;
    }
    h[nq] = run;
    ABX_CHECK_CUDA(cudaMemcpy(rowptr_user, h.data(), (nq + 1) * 8, cudaMemcpyDefault));
    if (cols_user) {
      ABX_REQUIRE(cap >= run, ABX_ERR_CAPACITY, "cols capacity %lld < nnz %lld", (long long)cap,
                  (long long)run);
      DevBuf<int64_t> rp, rpk;
      DevBuf<int32_t> colsd;
      DevBuf<double> dxd;
      ABX_TRY(rp.reserve(nq));
      ABX_TRY(rpk.reserve(nq));
      ABX_TRY(colsd.reserve(run ? run : 1));
      if (dx_user) {
        ABX_TRY(dxd.reserve((size_t)(run ? run : 1) * D));
        P.dx_out = dxd.ptr;
      }
      ABX_CHECK_CUDA(cudaMemcpyAsync(rp.ptr, h.data(), nq * 8, cudaMemcpyHostToDevice, s));
      k_rowptr_to_kernel<<<ceil_div(nq, TPB), TPB, 0, s>>>(rp.ptr, L.rows->perm.ptr, nq, rpk.ptr);
      ABX_CHECK_CUDA(cudaGetLastError());
      P.rowptr = rpk.ptr;
      P.cols_out = colsd.ptr;
      if (p->n > 0 && run > 0) ABX_TRY(launch_search<POL_LIST>(ctx, P));
      ABX_CHECK_CUDA(cudaMemcpyAsync(cols_user, colsd.ptr, run * 4, cudaMemcpyDefault, s));
      if (dx_user && run)
        ABX_CHECK_CUDA(cudaMemcpyAsync(dx_user, dxd.ptr, (size_t)run * D * 8, cudaMemcpyDefault, s));
      ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    }
  }
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

// Storage-order CSR of the neighbour lists of a particle set with itself at
// radius r (device arrays; used by the exact least-squares SPAI rows).
int self_csr_device(abx_particles *p, double r, DevBuf<int64_t> &rowptr, DevBuf<int32_t> &cols,
                    int64_t &nnz) {
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = p->n;
  PairLayout L;
  ABX_TRY(layout_build(ctx, p, r, nullptr, n, n, L));
  ABX_TRY(rowptr.reserve(n + 1));
  DevBuf<int32_t> cnt_k;
  ABX_TRY(cnt_k.reserve(n + 1));
  KParams P = base_params(L);
  P.kind = ABX_K_CONST;
  P.counts = cnt_k.ptr;
  ABX_CHECK_CUDA(cudaMemsetAsync(cnt_k.ptr, 0, (n + 1) * 4, s));
  if (n > 0) ABX_TRY(launch_pairs<POL_COUNT, ABX_K_CONST>(ctx, P, true));
  DevBuf<int64_t> rc;
  ABX_TRY(rc.reserve(n + 1));
  if (n) k_count_to_i64<<<ceil_div(n, TPB), TPB, 0, s>>>(cnt_k.ptr, L.rows->perm.ptr, n, rc.ptr);
  std::vector<int64_t> h(n + 1);
  if (n) ABX_CHECK_CUDA(cudaMemcpyAsync(h.data(), rc.ptr, n * 8, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  int64_t run = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t c = h[i];
    h[i] = run;
    run += c;
  }
  h[n] = run;
  nnz = run;
  ABX_CHECK_CUDA(cudaMemcpy(rowptr.ptr, h.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
  ABX_TRY(cols.reserve(run + 1));
  if (n > 0 && run > 0) {
    DevBuf<int64_t> rpk;
    ABX_TRY(rpk.reserve(n));
    k_rowptr_to_kernel<<<ceil_div(n, TPB), TPB, 0, s>>>(rowptr.ptr, L.rows->perm.ptr, n, rpk.ptr);
    P.rowptr = rpk.ptr;
    P.cols_out = cols.ptr;
    ABX_TRY(launch_pairs<POL_LIST, ABX_K_CONST>(ctx, P, true));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  return ABX_OK;
}

namespace {
constexpr int KNN_MAX = 64;

// k nearest neighbours (FP64 distance with periodic images, ties broken by
// storage index) of every particle of the layout's column set, by rings of
// fine cells around the particle's anchor cell.  One thread per particle.
__global__ void k_knn(KParams P, int k, int64_t n, int32_t *__restrict__ idx_out,
                      double *__restrict__ d2_out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const FineGrid &fg = P.fg;
  double bd[KNN_MAX];
  int bi[KNN_MAX];
  int cnt = 0;
  const int4 qc = P.qcell[q];
  const D4 xq = P.qpos[q];
  const int c[3] = {qc.x, qc.y, qc.z};
  const double qx[3] = {xq.x, xq.y, xq.z};
  double hmin = 1e300;
  int Rmax = 0;
  for (int e = 0; e < 3; ++e) {
    if (e < fg.eoff) continue;
    hmin = fmin(hmin, fg.h[e]);
    Rmax = max(Rmax, fg.m[e]);
  }
  for (int R = 0; R <= Rmax; ++R) {
    for (int o0 = -R; o0 <= R; ++o0) {
      if (fg.m[0] == 1 && o0 != 0) continue;
      for (int o1 = -R; o1 <= R; ++o1) {
        if (fg.m[1] == 1 && o1 != 0) continue;
        const bool edge01 = (abs(o0) == R) || (abs(o1) == R);
        for (int o2 = -R; o2 <= R; o2 += (edge01 ? 1 : max(2 * R, 1))) {
          int u[3] = {c[0] + o0, c[1] + o1, c[2] + o2}, img[3] = {0, 0, 0};
          bool ok = true;
          for (int e = 0; e < 3; ++e) {
            if (u[e] >= 0 && u[e] < fg.m[e]) continue;
            if (!fg.periodic[e] || u[e] < -fg.m[e] || u[e] >= 2 * fg.m[e]) { ok = false; break; }
            if (u[e] < 0) { u[e] += fg.m[e]; img[e] = 1; } else { u[e] -= fg.m[e]; img[e] = -1; }
          }
          if (!ok) continue;
          const uint32_t cell = ((uint32_t)u[0] * fg.m[1] + u[1]) * fg.m[2] + u[2];
          const uint32_t b = P.cell_start[cell], e = P.cell_start[cell + 1];
          for (uint32_t j = b; j < e; ++j) {
            const double d2 = exact_d2(xq, P.cpos[j], img, fg);
            const int sj = (int)P.cperm[j];
            if (cnt == k && (d2 > bd[k - 1] || (d2 == bd[k - 1] && sj > bi[k - 1]))) continue;
            int pos = cnt < k ? cnt++ : k - 1;
            while (pos > 0 && (bd[pos - 1] > d2 || (bd[pos - 1] == d2 && bi[pos - 1] > sj))) {
              bd[pos] = bd[pos - 1];
              bi[pos] = bi[pos - 1];
              --pos;
            }
            bd[pos] = d2;
            bi[pos] = sj;
          }
        }
      }
    }
    // every point of ring R+1 or beyond is at least R*h away
    const double reach = fmax(R * hmin * (1.0 - 1e-9), 0.0);
    if (cnt == k && bd[k - 1] <= reach * reach) break;
  }
  const int64_t row = P.cperm[q];
  for (int j = 0; j < k; ++j) {
    idx_out[row * k + j] = j < cnt ? bi[j] : -1;
    if (d2_out) d2_out[row * k + j] = j < cnt ? bd[j] : -1.0;
  }
  (void)qx;
}
}  // namespace

int knn_device(abx_particles *p, int k, int32_t *idx, double *d2) {
  abx_context *ctx = p->ctx;
  ABX_REQUIRE(k >= 1 && k <= KNN_MAX, ABX_ERR_INVALID, "k must be in 1..%d", KNN_MAX);
  GridDesc g;
  ABX_TRY(particles_grid_desc(p, &g));
  const int64_t n = p->n;
  if (n == 0) return ABX_OK;
  double vol = 1.0;
  for (int d = 0; d < p->dim; ++d) vol *= g.hi[d] - g.lo[d];
  const double h = std::pow(std::max(1.0, k / 4.0) * vol / (double)n, 1.0 / p->dim);
  PairLayout L;
  ABX_TRY(layout_build(ctx, p, 3.0 * h, nullptr, n, n, L));
  KParams P = base_params(L);
  k_knn<<<ceil_div(n, 128), 128, 0, ctx->stream>>>(P, k, n, idx, d2);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return ABX_OK;
}

}  // namespace abx

using namespace abx;

extern "C" {

int abx_radius_count(abx_particles *p, int64_t nq, const double *q, double r, int32_t *counts) {
  return abx_radius_count_lnorm(p, nq, q, r, 2, counts);
}

int abx_radius_query_csr(abx_particles *p, int64_t nq, const double *q, double r, int64_t *rowptr,
                         int32_t *cols, int64_t cap) {
  return abx_radius_query_csr_lnorm(p, nq, q, r, 2, rowptr, cols, cap);
}

int abx_radius_query_csr_dx(abx_particles *p, int64_t nq, const double *q, double r,
                            int64_t *rowptr, int32_t *cols, double *dx, int64_t cap) {
  ABX_REQUIRE(p && (q || nq == 0) && rowptr, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  return radius_query(p, nq, q, r, nullptr, rowptr, cols, cap, 2, cols ? dx : nullptr);
}

int abx_radius_count_lnorm(abx_particles *p, int64_t nq, const double *q, double r, int lnorm,
                           int32_t *counts) {
  ABX_REQUIRE(p && (q || nq == 0) && (counts || nq == 0), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  return radius_query(p, nq, q, r, counts, nullptr, nullptr, 0, lnorm);
}

int abx_radius_query_csr_lnorm(abx_particles *p, int64_t nq, const double *q, double r, int lnorm,
                               int64_t *rowptr, int32_t *cols, int64_t cap) {
  ABX_REQUIRE(p && (q || nq == 0) && rowptr, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  return radius_query(p, nq, q, r, nullptr, rowptr, cols, cap, lnorm);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Searches in a linearly transformed coordinate system (euclidean_search with
// a LinearTransform / ScaleTransform, src/Transform.h, src/Search.h:438-445):
// a particle is a neighbour iff !(|T dx|^2 > r^2), dx = x_j - (x + image*L).
// The candidates come from the ordinary search at radius r / sigma_min(T)
// (every point with |T dx| <= r has |dx| <= r / sigma_min), widened by 1e-9
// relative; the transformed test then runs on the device per candidate.
namespace abx {
namespace {
struct TMat {
  double m[9];  // row-major D x D
};

// (T dx)_i = ((T_i0 dx_0 + T_i1 dx_1) + T_i2 dx_2); accum = ((0 + y_0^2) + y_1^2) + y_2^2
__device__ __forceinline__ bool tf_inside(const double *dx, int D, const TMat &T, double r2,
                                          double *y) {
  double acc = 0.0;
  for (int i = 0; i < D; ++i) {
    double v = 0.0;
    for (int k = 0; k < D; ++k) v = __dadd_rn(v, __dmul_rn(T.m[i * D + k], dx[k]));
    y[i] = v;
    acc = __dadd_rn(acc, __dmul_rn(v, v));
  }
  return !(acc > r2);
}

__global__ void k_tf_count(const int64_t *__restrict__ rp, const double *__restrict__ dx,
                           int64_t nq, int D, TMat T, double r2, int64_t *__restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  int64_t c = 0;
  double y[3];
  for (int64_t e = rp[i]; e < rp[i + 1]; ++e) c += tf_inside(dx + e * D, D, T, r2, y) ? 1 : 0;
  cnt[i] = c;
}

__global__ void k_tf_fill(const int64_t *__restrict__ rp, const int32_t *__restrict__ cols,
                          const double *__restrict__ dx, int64_t nq, int D, TMat T, double r2,
                          const int64_t *__restrict__ orp, int32_t *__restrict__ ocols,
                          double *__restrict__ odx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  int64_t o = orp[i];
  double y[3];
  for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
    if (!tf_inside(dx + e * D, D, T, r2, y)) continue;
    ocols[o] = cols[e];
    if (odx)
      for (int d = 0; d < D; ++d) odx[o * D + d] = y[d];
    ++o;
  }
}

// smallest singular value of the D x D matrix T: the square root of the
// smallest eigenvalue of T^T T, by cyclic Jacobi rotations
double sigma_min(const double *T, int D) {
  double A[3][3] = {};
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j)
      for (int k = 0; k < D; ++k) A[i][j] += T[k * D + i] * T[k * D + j];
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < D; ++i)
      for (int j = i + 1; j < D; ++j) off += A[i][j] * A[i][j];
    if (off <= 1e-300) break;
    for (int p = 0; p < D; ++p)
      for (int q = p + 1; q < D; ++q) {
        if (A[p][q] == 0.0) continue;
        const double th = 0.5 * (A[q][q] - A[p][p]) / A[p][q];
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < D; ++k) {  // A <- A J
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < D; ++k) {  // A <- J^T A
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
      }
  }
  double lmin = A[0][0];
  for (int i = 1; i < D; ++i) lmin = std::min(lmin, A[i][i]);
  return lmin > 0 ? std::sqrt(lmin) : 0.0;
}
}  // namespace
}  // namespace abx

// Unique pairs within r of one particle set: the pairs a sweep over
// neighbouring buckets visits (bucket_pair_iterator, src/Search.h:498-764,
// together with the pairs inside each bucket), each once -- (i, j) with i < j
// in storage order, dx = x_j - (x_i + image*L) of the accepted image and
// !(|dx|^2 > r^2) -- from the self search's CSR, filtered on the device.
namespace abx {
namespace {
__global__ void k_soa_to_aos(const double *__restrict__ soa, int64_t n, int dim,
                             double *__restrict__ aos) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int d = 0; d < dim; ++d) aos[i * dim + d] = soa[(int64_t)d * n + i];
}

__global__ void k_upper_count(const int64_t *__restrict__ rp, const int32_t *__restrict__ cols,
                              int64_t n, int64_t *__restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t c = 0;
  for (int64_t e = rp[i]; e < rp[i + 1]; ++e) c += cols[e] > i ? 1 : 0;
  cnt[i] = c;
}

__global__ void k_upper_fill(const int64_t *__restrict__ rp, const int32_t *__restrict__ cols,
                             const double *__restrict__ dx, int64_t n, int D,
                             const int64_t *__restrict__ orp, int32_t *__restrict__ oi,
                             int32_t *__restrict__ oj, double *__restrict__ odx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t o = orp[i];
  for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
    if (cols[e] <= i) continue;
    oi[o] = (int32_t)i;
    oj[o] = cols[e];
    if (odx)
      for (int d = 0; d < D; ++d) odx[o * D + d] = dx[e * D + d];
    ++o;
  }
}
}  // namespace
}  // namespace abx

extern "C" int abx_radius_pairs(abx_particles *p, double r, int64_t *npairs, int32_t *pi,
                                int32_t *pj, double *dx, int64_t cap) {
  ABX_REQUIRE(p && npairs, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(r >= 0 && std::isfinite(r), ABX_ERR_INVALID, "invalid radius");
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called on this particle set");
  ABX_TRY(ctx_activate(p->ctx));
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = p->n;
  const int D = p->dim;
  *npairs = 0;
  if (n == 0) return ABX_OK;
  DevBuf<double> aos;
  ABX_TRY(aos.reserve((size_t)n * D));
  k_soa_to_aos<<<ceil_div(n, TPB), TPB, 0, s>>>(p->pos.ptr, n, D, aos.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  std::vector<int64_t> hc(n + 1);
  ABX_TRY(radius_query(p, n, aos.ptr, r, nullptr, hc.data(), nullptr, 0, 2));
  const int64_t nc = hc[n];
  DevBuf<int64_t> crp, cnt, orp;
  DevBuf<int32_t> ccols;
  DevBuf<double> cdx;
  ABX_TRY(crp.reserve(n + 1));
  ABX_TRY(cnt.reserve(n + 1));
  ABX_TRY(ccols.reserve(nc + 1));
  if (dx) ABX_TRY(cdx.reserve((size_t)(nc + 1) * D));
  ABX_TRY(radius_query(p, n, aos.ptr, r, nullptr, crp.ptr, ccols.ptr, nc, 2,
                       dx ? cdx.ptr : nullptr));
  k_upper_count<<<ceil_div(n, TPB), TPB, 0, s>>>(crp.ptr, ccols.ptr, n, cnt.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  std::vector<int64_t> h(n + 1);
  ABX_CHECK_CUDA(cudaMemcpyAsync(h.data(), cnt.ptr, n * 8, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  int64_t run = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t c = h[i];
    h[i] = run;
    run += c;
  }
  h[n] = run;
  *npairs = run;
  if (!pi) return ABX_OK;
  ABX_REQUIRE(pj, ABX_ERR_INVALID, "pi and pj are both given or both NULL");
  ABX_REQUIRE(cap >= run, ABX_ERR_CAPACITY, "pair capacity %lld < %lld pairs", (long long)cap,
              (long long)run);
  DevBuf<int32_t> oi, oj;
  DevBuf<double> odx;
  ABX_TRY(oi.reserve(run + 1));
  ABX_TRY(oj.reserve(run + 1));
  if (dx) ABX_TRY(odx.reserve((size_t)(run + 1) * D));
  ABX_TRY(orp.reserve(n + 1));
  ABX_CHECK_CUDA(cudaMemcpyAsync(orp.ptr, h.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s));
  k_upper_fill<<<ceil_div(n, TPB), TPB, 0, s>>>(crp.ptr, ccols.ptr, dx ? cdx.ptr : nullptr, n, D,
                                                orp.ptr, oi.ptr, oj.ptr, dx ? odx.ptr : nullptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  if (run) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(pi, oi.ptr, run * 4, cudaMemcpyDefault, s));
    ABX_CHECK_CUDA(cudaMemcpyAsync(pj, oj.ptr, run * 4, cudaMemcpyDefault, s));
    if (dx) ABX_CHECK_CUDA(cudaMemcpyAsync(dx, odx.ptr, (size_t)run * D * 8, cudaMemcpyDefault, s));
  }
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

extern "C" int abx_radius_query_csr_transform(abx_particles *p, int64_t nq, const double *q,
                                              double r, const double *T, int64_t *rowptr,
                                              int32_t *cols, double *dx, int64_t cap) {
  ABX_REQUIRE(p && (q || nq == 0) && rowptr && T, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(r >= 0 && std::isfinite(r), ABX_ERR_INVALID, "invalid radius");
  ABX_TRY(ctx_activate(p->ctx));
  const int D = p->dim;
  TMat tm{};
  for (int k = 0; k < D * D; ++k) {
    ABX_REQUIRE(std::isfinite(T[k]), ABX_ERR_INVALID, "transform entries must be finite");
    tm.m[k] = T[k];
  }
  const double smin = sigma_min(T, D);
  ABX_REQUIRE(smin > 0 && std::isfinite(r / smin), ABX_ERR_INVALID,
              "the transform must be invertible (smallest singular value %g)", smin);
  const double R = r / smin * (1.0 + 1e-9);
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  // candidates: CSR with the accepted image's dx, on the device
  std::vector<int64_t> hc(nq + 1);
  ABX_TRY(radius_query(p, nq, q, R, nullptr, hc.data(), nullptr, 0, 2));
  const int64_t nc = hc[nq];
  DevBuf<int64_t> crp, cnt, orp;
  DevBuf<int32_t> ccols;
  DevBuf<double> cdx;
  ABX_TRY(crp.reserve(nq + 1));
  ABX_TRY(cnt.reserve(nq + 1));
  ABX_TRY(ccols.reserve(nc + 1));
  ABX_TRY(cdx.reserve((size_t)(nc + 1) * D));
  ABX_TRY(radius_query(p, nq, q, R, nullptr, crp.ptr, ccols.ptr, nc, 2, cdx.ptr));
  if (nq)
    k_tf_count<<<ceil_div(nq, TPB), TPB, 0, s>>>(crp.ptr, cdx.ptr, nq, D, tm, r * r, cnt.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  std::vector<int64_t> h(nq + 1);
  if (nq) ABX_CHECK_CUDA(cudaMemcpyAsync(h.data(), cnt.ptr, nq * 8, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  int64_t run = 0;
  for (int64_t i = 0; i < nq; ++i) {
    const int64_t c = h[i];
    h[i] = run;
    run += c;
  }
  h[nq] = run;
  ABX_CHECK_CUDA(cudaMemcpy(rowptr, h.data(), (nq + 1) * 8, cudaMemcpyDefault));
  if (!cols) return ABX_OK;
  ABX_REQUIRE(cap >= run, ABX_ERR_CAPACITY, "cols capacity %lld < nnz %lld", (long long)cap,
              (long long)run);
  DevBuf<int32_t> ocols;
  DevBuf<double> odx;
  ABX_TRY(ocols.reserve(run + 1));
  if (dx) ABX_TRY(odx.reserve((size_t)(run + 1) * D));
  ABX_TRY(orp.reserve(nq + 1));
  ABX_CHECK_CUDA(cudaMemcpyAsync(orp.ptr, h.data(), (nq + 1) * 8, cudaMemcpyHostToDevice, s));
  if (nq)
    k_tf_fill<<<ceil_div(nq, TPB), TPB, 0, s>>>(crp.ptr, ccols.ptr, cdx.ptr, nq, D, tm, r * r,
                                                 orp.ptr, ocols.ptr, dx ? odx.ptr : nullptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  if (run) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(cols, ocols.ptr, run * 4, cudaMemcpyDefault, s));
    if (dx) ABX_CHECK_CUDA(cudaMemcpyAsync(dx, odx.ptr, (size_t)run * D * 8, cudaMemcpyDefault, s));
  }
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free sparse matvec (abx_operator_matvec_noalloc).
//
// Some callers cannot call cudaMalloc while they apply an operator: code that
// runs under a device-memory budget owned by another runtime (a framework
// with its own caching allocator, a solver embedded in a simulation that
// pre-sizes everything at start-up), or a time-stepping loop that must not
// pay cudaMalloc/cudaFree's implicit device-wide synchronisation.  For them
// this entry point keeps the per-call scratch of the sparse matvec -- b
// gathered into the operator's internal order, the result before it is
// scattered back to storage order, and the work counter of the pair kernel
// -- in one file-scope device array of fixed size instead of in buffers
// owned by the operator.  Every GPU that loads the library holds this array
// until the process exits.
namespace abx {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20;  // 32 MiB
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on `device` (current), looked up once
// per device.  In host code the symbol itself is only a host-side stand-in,
// so kernels must be given this address, never the symbol.
int noalloc_scratch(int device, unsigned char **out) {
  ABX_REQUIRE(device >= 0 && device < NOALLOC_MAX_DEVICES, ABX_ERR_INVALID,
              "device %d beyond the allocation-free entry point's table", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[device]) {
    void *p = nullptr;
    ABX_CHECK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[device] = (unsigned char *)p;
  }
  *out = g_noalloc_addr[device];
  return ABX_OK;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace
}  // namespace abx

extern "C" int abx_operator_matvec_noalloc(abx_operator *op, const double *b, double *c) {
  ABX_REQUIRE(op, ABX_ERR_INVALID, "null operator");
  ABX_REQUIRE(op->kind == 0, ABX_ERR_INVALID,
              "abx_operator_matvec_noalloc: only sparse operators are supported");
  const int64_t nr = op->rows->n, nc = op->cols->n;
  ABX_REQUIRE((b || nc == 0) && (c || nr == 0), ABX_ERR_INVALID, "null vector");
  abx_context *ctx = op->rows->ctx;
  ABX_TRY(ctx_activate(ctx));
  ABX_REQUIRE(op->cols->searchable, ABX_ERR_STATE,
              "init_neighbour_search not called on the column particle set");
  // A stale layout would have to be rebuilt, which allocates: refuse.
  ABX_REQUIRE(op->pairs && op->pairs->cols_version == op->cols->version &&
                  op->pairs->rows_version == op->rows->version,
              ABX_ERR_STATE,
              "abx_operator_matvec_noalloc: the particle sets changed since the operator was "
              "built; rebuild it (or call abx_operator_matvec once) before calling this");
  ABX_REQUIRE((nc == 0 || device_ptr_usable(b, ctx->device) == 1) &&
                  (nr == 0 || device_ptr_usable(c, ctx->device) == 1),
              ABX_ERR_INVALID,
              "abx_operator_matvec_noalloc: b and c must be device memory of the context's "
              "GPU (host vectors would need staging buffers)");
  if (nr == 0) return ABX_OK;
  const bool mixed = op->precision == ABX_PREC_MIXED && op->k.kind != ABX_K_SCALAR_SUM;
  const size_t need = align256((size_t)nc * (mixed ? sizeof(float) : sizeof(double))) +
                      align256((size_t)nr * sizeof(double)) + 256;
  ABX_REQUIRE(need <= NOALLOC_SCRATCH_BYTES, ABX_ERR_CAPACITY,
              "abx_operator_matvec_noalloc: needs %zu bytes of scratch (%lld rows, %lld "
              "columns) but the fixed array holds %zu bytes",
              need, (long long)nr, (long long)nc, NOALLOC_SCRATCH_BYTES);
  unsigned char *base = nullptr;
  ABX_TRY(noalloc_scratch(ctx->device, &base));
  const size_t bbytes = align256((size_t)nc * (mixed ? sizeof(float) : sizeof(double)));
  void *bk = base;
  double *ck = (double *)(base + bbytes);
  int *counter = (int *)(base + bbytes + align256((size_t)nr * sizeof(double)));
  cudaStream_t s = ctx->stream;
  PairLayout &L = *op->pairs;
  if (nc == 0) {
    ABX_CHECK_CUDA(cudaMemsetAsync(c, 0, nr * sizeof(double), s));
    return ABX_OK;
  }
  k_gather_b<<<ceil_div(nc, TPB), TPB, 0, s>>>(b, L.cols.perm.ptr, nc,
                                               mixed ? (float *)bk : nullptr,
                                               mixed ? nullptr : (double *)bk);
  ABX_CHECK_CUDA(cudaGetLastError());
  KParams P = base_params(L);
  P.kind = op->k.kind;
  P.p0 = op->k.p[0];
  P.p0f = (float)op->k.p[0];
  P.c_exp2 = (float)(-op->k.p[0] * 1.4426950408889634);
  P.b32 = mixed ? (const float *)bk : nullptr;
  P.b64 = mixed ? nullptr : (const double *)bk;
  P.s_col = L.sk.ptr;
  P.s_row = L.sq.ptr;
  P.c = ck;
  P.counter = counter;  // zeroed by the launch helper before every launch
  ABX_TRY(launch_pairs_kind<POL_MATVEC>(ctx, P, mixed));
  k_scatter_c<<<ceil_div(nr, TPB), TPB, 0, s>>>(ck, L.rows->perm.ptr, nr, c);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

extern "C" int abx_knn(abx_particles *p, int k, int32_t *idx, double *d2) {
  ABX_REQUIRE(p && (idx || p->n == 0), ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called on this particle set");
  ABX_TRY(ctx_activate(p->ctx));
  const int64_t n = p->n;
  HostStage si, sd;
  void *di, *dd = nullptr;
  ABX_TRY(si.out(p->ctx, idx, (size_t)n * k * 4, &di));
  if (d2) ABX_TRY(sd.out(p->ctx, d2, (size_t)n * k * 8, &dd));
  ABX_TRY(knn_device(p, k, (int32_t *)di, (double *)dd));
  ABX_TRY(si.finish(p->ctx, idx, (size_t)n * k * 4));
  if (d2) ABX_TRY(sd.finish(p->ctx, d2, (size_t)n * k * 8));
  return ABX_OK;
}
