// Particle storage and the CellListOrdered build on the GPU.
//
// Reference flow restated here (Particles::init_neighbour_search,
// src/Particles.h:445-456):
//   set_domain -> set_domain_impl (grid, with the 2x hysteresis on n,
//                 src/CellListOrdered.h:132-186)
//   update_positions (src/NeighbourSearchBase.h:350-495):
//     enforce_domain_lambda (:185-238)       -> k_enforce_domain
//     exclusive_scan(alive) + scatter_if     -> exclusive_scan_u32 + k_compact
//     update_positions_impl (CellListOrdered.h:190-259):
//       transform(pos -> bucket index)       -> k_hash
//       sort_by_key (stable, as Thrust)      -> radix_sort_pairs
//       lower_bound / upper_bound per bucket -> k_count_cells + scan
//   Particles::reorder (src/Particles.h:694-726) -> k_gather_*
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "handles.cuh"

namespace abx {

namespace {

constexpr int TPB = 256;

__global__ void k_enforce_domain(double *__restrict__ pos, int64_t n, int dim, GridDesc g,
                                 uint32_t *__restrict__ alive) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t a = 1;
  for (int d = 0; d < dim; ++d) {
    double r = pos[(int64_t)d * n + i];
    if (!isfinite(r)) {
      a = 0;
    } else if (g.periodic[d]) {
      while (r < g.lo[d]) r = __dadd_rn(r, __dsub_rn(g.hi[d], g.lo[d]));
      while (r >= g.hi[d]) r = __dsub_rn(r, __dsub_rn(g.hi[d], g.lo[d]));
    } else if ((r < g.lo[d]) || (r >= g.hi[d])) {
      a = 0;
    }
    pos[(int64_t)d * n + i] = r;
  }
  alive[i] = a;
}

__global__ void k_compact(const uint32_t *__restrict__ alive, const uint32_t *__restrict__ scan,
                          int64_t n, uint32_t *__restrict__ idx) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (alive[i]) idx[scan[i]] = (uint32_t)i;
}

// point_to_bucket_index::find_bucket_index (src/detail/SpatialUtil.h:125-138):
// v_d = (int)floor((r_d - bmin_d) * inv_side_d), collapsed with the last
// dimension fastest in unsigned 32-bit arithmetic.
__device__ __forceinline__ uint32_t bucket_key(const double *x, const GridDesc &g) {
  uint32_t key = 0, mult = 1;
  for (int d = g.dim - 1; d >= 0; --d) {
    if (d != g.dim - 1) mult *= g.size[d + 1];
    const int v = (int)floor(__dmul_rn(__dsub_rn(x[d], g.lo[d]), g.inv_side[d]));
    key += mult * (uint32_t)v;
  }
  return key;
}

// point_to_tag (src/detail/SpatialUtil.h:255-286): per level, one bit per
// dimension (dimension 0 most significant) from p < mid, bisecting the box.
__global__ void k_tag(const double *__restrict__ pos, int64_t n, GridDesc g, int max_level,
                      const uint32_t *__restrict__ idx, int64_t na, uint32_t *__restrict__ keys,
                      uint32_t *__restrict__ vals) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= na) return;
  const uint32_t i = idx[k];
  double p[3], bmin[3], bmax[3];
  for (int d = 0; d < g.dim; ++d) {
    p[d] = pos[(int64_t)d * n + i];
    bmin[d] = g.lo[d];
    bmax[d] = g.hi[d];
  }
  int result = 0;
  for (int level = 1; level <= max_level; ++level) {
    int hh[3];
    double mid[3];
    for (int d = 0; d < g.dim; ++d) {
      mid[d] = __dmul_rn(0.5, __dadd_rn(bmin[d], bmax[d]));
      hh[d] = (p[d] < mid[d]) ? 0 : 1;
      result |= hh[d];
      result <<= 1;
    }
    for (int d = 0; d < g.dim; ++d) {
      if (hh[d]) bmin[d] = mid[d]; else bmax[d] = mid[d];
    }
  }
  result >>= 1;
  keys[k] = (uint32_t)result;
  vals[k] = i;
}

__global__ void k_hash(const double *__restrict__ pos, int64_t n, GridDesc g,
                       const uint32_t *__restrict__ idx, int64_t na, uint32_t *__restrict__ keys,
                       uint32_t *__restrict__ vals) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= na) return;
  const uint32_t i = idx[k];
  double x[3] = {0, 0, 0};
  for (int d = 0; d < g.dim; ++d) x[d] = pos[(int64_t)d * n + i];
  keys[k] = bucket_key(x, g);
  vals[k] = i;
}

// Marks each bucket's run in the sorted keys: first[key] = start, last[key] =
// one past the end (both zero for empty buckets).  lower_bound/upper_bound of
// the reference (src/CellListOrdered.h:231-239) then follow from a scan of the
// run lengths.
__global__ void k_mark_runs(const uint32_t *__restrict__ keys, int64_t na, uint32_t ncells,
                            uint32_t *__restrict__ first, uint32_t *__restrict__ last) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= na) return;
  const uint32_t key = keys[k];
  if (key >= ncells) return;
  if (k == 0 || keys[k - 1] != key) first[key] = (uint32_t)k;
  if (k == na - 1 || keys[k + 1] != key) last[key] = (uint32_t)(k + 1);
}

__global__ void k_run_length(const uint32_t *__restrict__ first, uint32_t ncells,
                             uint32_t *__restrict__ last_to_count) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  last_to_count[c] -= first[c];
}

__global__ void k_bucket_end(const uint32_t *__restrict__ begin, const uint32_t *__restrict__ counts,
                             uint32_t ncells, uint32_t *__restrict__ end) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  end[c] = begin[c] + counts[c];
}

__global__ void k_gather_pos(const double *__restrict__ src, int64_t n, int dim,
                             const uint32_t *__restrict__ perm, int64_t na,
                             double *__restrict__ dst) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= na) return;
  const uint32_t i = perm[k];
  for (int d = 0; d < dim; ++d) dst[(int64_t)d * na + k] = src[(int64_t)d * n + i];
}

template <class T>
__global__ void k_gather(const T *__restrict__ src, const uint32_t *__restrict__ perm, int64_t na,
                         T *__restrict__ dst) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= na) return;
  dst[k] = src[perm[k]];
}

// new particles (AoS) into rows [n0, n) of SoA columns of stride n
__global__ void k_append_aos(const double *__restrict__ aos, int64_t n_new, int dim, int64_t n0,
                             int64_t n, double *__restrict__ soa) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_new) return;
  for (int d = 0; d < dim; ++d) soa[(int64_t)d * n + n0 + i] = aos[i * dim + d];
}

__global__ void k_mark_dead(double *__restrict__ pos, int64_t first, int64_t last) {
  int64_t i = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < last) pos[i] = __longlong_as_double(0x7ff8000000000000ll);  // NaN
}

// one 32-bit half of each id (as unsigned 64-bit), in the order `order`
// (null: storage order); vals get the storage index
__global__ void k_id_half(const int64_t *__restrict__ ids, const uint32_t *__restrict__ order,
                          int64_t n, int high, uint32_t *__restrict__ keys,
                          uint32_t *__restrict__ vals) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = order ? order[k] : (uint32_t)k;
  const uint64_t id = (uint64_t)ids[i];
  keys[k] = high ? (uint32_t)(id >> 32) : (uint32_t)id;
  vals[k] = i;
}

__global__ void k_idmap_fill(const int64_t *__restrict__ ids, const uint32_t *__restrict__ perm,
                             int64_t n, int64_t *__restrict__ key, uint32_t *__restrict__ val) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  key[k] = ids[perm[k]];
  val[k] = perm[k];
}

// find_id_map (src/NeighbourSearchBase.h:276-281): lower_bound of the id in
// the sorted keys; storage index, or -1 when the id is not in the set
__global__ void k_find_ids(const int64_t *__restrict__ key, const uint32_t *__restrict__ val,
                           int64_t n, const int64_t *__restrict__ q, int64_t nq,
                           int64_t *__restrict__ out) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  const uint64_t id = (uint64_t)q[t];
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if ((uint64_t)key[mid] < id) lo = mid + 1; else hi = mid;
  }
  out[t] = (lo < n && (uint64_t)key[lo] == id) ? (int64_t)val[lo] : -1;
}

__global__ void k_aos_to_soa(const double *__restrict__ aos, int64_t n, int dim,
                             double *__restrict__ soa) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int d = 0; d < dim; ++d) soa[(int64_t)d * n + i] = aos[i * dim + d];
}

__global__ void k_soa_to_aos(const double *__restrict__ soa, int64_t n, int dim,
                             double *__restrict__ aos) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int d = 0; d < dim; ++d) aos[i * dim + d] = soa[(int64_t)d * n + i];
}

__global__ void k_iota64(int64_t *ids, int64_t n, int64_t start) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ids[i] = start + i;
}

}  // namespace

// set_domain_impl (src/CellListOrdered.h:132-186) as a function: the grid
// that alive count n leaves (recomputed only when n left [0.5, 2] x the count
// the current grid was computed with) and the count it then records.
GridDesc grid_for_count(const abx_particles *p, size_t n, size_t *calc_n) {
  GridDesc g = p->grid;
  *calc_n = p->size_calculated_with_n;
  if (!(n < 0.5 * p->size_calculated_with_n || n > 2 * p->size_calculated_with_n)) return g;
  *calc_n = n;
  const int D = p->dim;
  if (p->n_leaf > (double)n) {
    for (int d = 0; d < D; ++d) g.size[d] = 1;
  } else {
    double total_volume = 1.0;
    for (int d = 0; d < D; ++d) total_volume *= (g.hi[d] - g.lo[d]);
    const double box_volume = p->n_leaf / double(n) * total_volume;
    const double box_side = std::pow(box_volume, 1.0 / D);
    for (int d = 0; d < D; ++d) {
      g.size[d] = (unsigned int)std::floor((g.hi[d] - g.lo[d]) / box_side);
      if (g.size[d] == 0) g.size[d] = 1;
    }
  }
  g.ncells = 1;
  for (int d = 0; d < D; ++d) {
    g.side[d] = (g.hi[d] - g.lo[d]) / g.size[d];
    g.inv_side[d] = 1.0 / g.side[d];
    g.ncells *= g.size[d];
  }
  for (int d = D; d < 3; ++d) {
    g.size[d] = 1;
    g.lo[d] = 0.0;
    g.hi[d] = 1.0;
    g.side[d] = 1.0;
    g.inv_side[d] = 1.0;
    g.periodic[d] = 0;
  }
  return g;
}

namespace {

// set_domain_impl applied to the particle set.  Returns true if the grid was
// recomputed.
bool set_domain_impl(abx_particles *p, size_t n) {
  const size_t before = p->size_calculated_with_n;
  const bool recompute = n < 0.5 * before || n > 2 * before;
  size_t calc = 0;
  p->grid = grid_for_count(p, n, &calc);
  p->size_calculated_with_n = calc;
  return recompute;
}

// HyperOctree::build_tree (src/OctTree.h:328-475) on the sorted tags.
void build_octree(abx_particles *p, const std::vector<int> &tags) {
  OctTree &T = p->tree;
  const int D = p->dim;
  const int nchild = 1 << D;
  T = OctTree();
  T.dim = D;
  T.max_level = 32 / D - 2;
  auto add = [&](int tag, int level, int b, int e, int kind, int parent) {
    T.tag.push_back(tag);
    T.level.push_back(level);
    T.begin.push_back(b);
    T.end.push_back(e);
    T.kind.push_back(kind);
    T.first_child.push_back(-1);
    T.parent.push_back(parent);
    return (int)T.tag.size() - 1;
  };
  add(0, 0, 0, (int)tags.size(), 2, -1);  // root
  std::vector<int> active(1, 0);
  for (int level = 1; !active.empty(); ++level) {
    const int shift = (T.max_level - level) * D;
    const int length = (1 << shift) - 1;
    std::vector<int> next;
    for (int a : active) {
      T.first_child[a] = (int)T.tag.size();
      for (int c = 0; c < nchild; ++c) {
        const int mask = T.tag[a] | (c << shift);
        const int lb = (int)(std::lower_bound(tags.begin(), tags.end(), mask) - tags.begin());
        const int ub =
            (int)(std::upper_bound(tags.begin(), tags.end(), mask + length) - tags.begin());
        const int count = ub - lb;
        int kind = 0;
        if (count > 0) kind = (level == T.max_level || count <= p->n_leaf) ? 1 : 2;
        const int id = add(mask, level, lb, ub, kind, a);
        if (kind == 1) T.leaves.push_back(id);
        if (kind == 2) next.push_back(id);
      }
    }
    active.swap(next);
  }
}

int update_positions(abx_particles *p) {
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = p->n;
  const int D = p->dim;
  p->searchable = false;
  ++p->version;
  if (n == 0) {
    if (p->search_kind == 1) {
      p->oct.reset();
      build_octree(p, std::vector<int>());
    }
    set_domain_impl(p, 0);
    p->n_alive_prev = 0;
    ABX_TRY(p->bucket_begin.reserve(p->grid.ncells));
    ABX_TRY(p->bucket_end.reserve(p->grid.ncells));
    ABX_CHECK_CUDA(cudaMemsetAsync(p->bucket_begin.ptr, 0, p->grid.ncells * 4, s));
    ABX_CHECK_CUDA(cudaMemsetAsync(p->bucket_end.ptr, 0, p->grid.ncells * 4, s));
    p->searchable = true;
    return ABX_OK;
  }
  ABX_REQUIRE(n < (int64_t)0xFFFFFFFFll, ABX_ERR_INVALID, "too many particles (%lld)",
              (long long)n);
  if (p->search_kind == 0) {
    ABX_TRY(celllist_build(p));
    p->searchable = true;
    return ABX_OK;
  }
  // HyperOctree:
  // scratch: alive(n) scan(n) idx(n) keys(n) vals(n) keys_alt(n) vals_alt(n) temp
  size_t off = 0;
  carve_size<uint32_t>(off, n);
  carve_size<uint32_t>(off, n);
  carve_size<uint32_t>(off, scan_temp_elems(n));
  carve_size<uint32_t>(off, n);
  carve_size<uint32_t>(off, n);
  carve_size<uint32_t>(off, n);
  carve_size<uint32_t>(off, n);
  carve_size<uint32_t>(off, radix_temp_u32(n));
  ABX_TRY(ctx->scratch.reserve(off + 256));
  unsigned char *base = ctx->scratch.ptr;
  off = 0;
  uint32_t *alive = carve<uint32_t>(base, off, n);
  uint32_t *scan = carve<uint32_t>(base, off, n);
  uint32_t *stmp = carve<uint32_t>(base, off, scan_temp_elems(n));
  uint32_t *vals = carve<uint32_t>(base, off, n);
  uint32_t *keys_alt = carve<uint32_t>(base, off, n);
  uint32_t *vals_alt = carve<uint32_t>(base, off, n);
  uint32_t *idx = carve<uint32_t>(base, off, n);
  uint32_t *rtmp = carve<uint32_t>(base, off, radix_temp_u32(n));

  GridDesc g = p->grid;
  k_enforce_domain<<<ceil_div(n, TPB), TPB, 0, s>>>(p->pos.ptr, n, D, g, alive);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_CHECK_CUDA(cudaMemcpyAsync(scan, alive, n * 4, cudaMemcpyDeviceToDevice, s));
  ABX_TRY(exclusive_scan_u32(scan, n, stmp, s));
  uint32_t last[2];
  ABX_CHECK_CUDA(cudaMemcpyAsync(&last[0], scan + n - 1, 4, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(&last[1], alive + n - 1, 4, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  const int64_t na = (int64_t)last[0] + last[1];
  k_compact<<<ceil_div(n, TPB), TPB, 0, s>>>(alive, scan, n, idx);
  ABX_CHECK_CUDA(cudaGetLastError());

  uint32_t *keys = nullptr;
  if (p->search_kind == 1) {
    // HyperOctree: tags, stable sort, tree built on the host from the tags.
    g = p->grid;
    const int max_level = 32 / D - 2;
    ABX_TRY(p->keys.reserve(na > 0 ? na : 1));
    keys = p->keys.ptr;
    if (na > 0) {
      k_tag<<<ceil_div(na, TPB), TPB, 0, s>>>(p->pos.ptr, n, g, max_level, idx, na, keys, vals);
      ABX_CHECK_CUDA(cudaGetLastError());
      ABX_TRY(radix_sort_pairs(keys, vals, na, max_level * D, keys_alt, vals_alt, rtmp, s));
    }
    if (na > 0) {
      ABX_TRY(octree_build_device(p, keys, na));
    } else {
      p->oct.reset();
      build_octree(p, std::vector<int>());
    }
  } else {
  set_domain_impl(p, (size_t)na);
  g = p->grid;
  ABX_TRY(p->keys.reserve(na > 0 ? na : 1));
  ABX_TRY(p->bucket_begin.reserve(g.ncells));
  ABX_TRY(p->bucket_end.reserve(g.ncells));
  keys = p->keys.ptr;
  if (na > 0) {
    k_hash<<<ceil_div(na, TPB), TPB, 0, s>>>(p->pos.ptr, n, g, idx, na, keys, vals);
    ABX_CHECK_CUDA(cudaGetLastError());
    // Every alive position satisfies lo <= x < hi, so v_d <= size_d and the
    // key is at most collapse(size): sort on that many bits.
    uint64_t maxkey = 0, mult = 1;
    for (int d = D - 1; d >= 0; --d) {
      if (d != D - 1) mult *= g.size[d + 1];
      maxkey += mult * (uint64_t)g.size[d];
    }
    int bits = 0;
    while (bits < 32 && (maxkey >> bits) != 0) ++bits;
    if (maxkey > 0xFFFFFFFFull) bits = 32;
    ABX_TRY(radix_sort_pairs(keys, vals, na, bits, keys_alt, vals_alt, rtmp, s));
  }
  // bucket runs -> counts -> begin (exclusive scan) -> end
  uint32_t *bb = p->bucket_begin.ptr, *be = p->bucket_end.ptr;
  ABX_CHECK_CUDA(cudaMemsetAsync(bb, 0, (size_t)g.ncells * 4, s));
  ABX_CHECK_CUDA(cudaMemsetAsync(be, 0, (size_t)g.ncells * 4, s));
  if (na > 0) {
    k_mark_runs<<<ceil_div(na, TPB), TPB, 0, s>>>(keys, na, g.ncells, bb, be);
    ABX_CHECK_CUDA(cudaGetLastError());
  }
  k_run_length<<<ceil_div(g.ncells, TPB), TPB, 0, s>>>(bb, g.ncells, be);
  ABX_CHECK_CUDA(cudaGetLastError());
  uint32_t *counts = be;
  ABX_CHECK_CUDA(cudaMemcpyAsync(bb, counts, (size_t)g.ncells * 4, cudaMemcpyDeviceToDevice, s));
  {
    const size_t need = scan_temp_elems(g.ncells);
    if (need > scan_temp_elems(n)) {
      DevBuf<uint32_t> extra;
      ABX_TRY(extra.reserve(need));
      ABX_TRY(exclusive_scan_u32(bb, g.ncells, extra.ptr, s));
      ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    } else {
      ABX_TRY(exclusive_scan_u32(bb, g.ncells, stmp, s));
    }
  }
  k_bucket_end<<<ceil_div(g.ncells, TPB), TPB, 0, s>>>(bb, counts, g.ncells, be);
  ABX_CHECK_CUDA(cudaGetLastError());

  }
  // reorder (gather) every column into cell order; dead particles are dropped
  ABX_TRY(p->pos_alt.reserve((size_t)D * (na > 0 ? na : 1)));
  ABX_TRY(p->ids_alt.reserve(na > 0 ? na : 1));
  if (na > 0) {
    k_gather_pos<<<ceil_div(na, TPB), TPB, 0, s>>>(p->pos.ptr, n, D, vals, na, p->pos_alt.ptr);
    k_gather<int64_t><<<ceil_div(na, TPB), TPB, 0, s>>>(p->ids.ptr, vals, na, p->ids_alt.ptr);
    if (p->has_scalar) {
      ABX_TRY(p->scalar_alt.reserve(na));
      k_gather<double><<<ceil_div(na, TPB), TPB, 0, s>>>(p->scalar.ptr, vals, na,
                                                         p->scalar_alt.ptr);
    }
    ABX_CHECK_CUDA(cudaGetLastError());
  }
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
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  p->searchable = true;
  return ABX_OK;
}

}  // namespace

void OctTree::box(const GridDesc &g, int node, double *lo, double *hi) const {
  for (int d = 0; d < dim; ++d) {
    lo[d] = g.lo[d];
    hi[d] = g.hi[d];
  }
  const int L = level[node], t = tag[node];
  for (int l = 1; l <= L; ++l) {
    for (int d = 0; d < dim; ++d) {
      const int bit = (t >> ((max_level - l) * dim + (dim - 1 - d))) & 1;
      const double mid = 0.5 * (lo[d] + hi[d]);
      if (bit) lo[d] = mid; else hi[d] = mid;
    }
  }
}

void particles_retain(abx_particles *p) { p->refs.fetch_add(1); }

void particles_release(abx_particles *p) {
  if (!p || p->refs.fetch_sub(1) != 1) return;
  abx_context *ctx = p->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete p;
  ctx_release(ctx);
}

int particles_grid_desc(const abx_particles *p, GridDesc *g) {
  ABX_REQUIRE(p && p->searchable, ABX_ERR_STATE,
              "init_neighbour_search not called on this particle set");
  *g = p->grid;
  return ABX_OK;
}

}  // namespace abx

using namespace abx;

extern "C" {

int abx_particles_create(abx_context *ctx, int dim, abx_particles **out) {
  ABX_REQUIRE(ctx && out, ABX_ERR_INVALID, "abx_particles_create: null argument");
  ABX_REQUIRE(dim >= 1 && dim <= 3, ABX_ERR_INVALID, "dimension %d not supported (1..3)", dim);
  abx_particles *p = new abx_particles();
  p->ctx = ctx;
  p->dim = dim;
  for (int d = 0; d < 3; ++d) {
    p->grid.size[d] = 1;
    p->grid.side[d] = 1.0;
    p->grid.inv_side[d] = 1.0;
  }
  p->grid.dim = dim;
  p->grid.ncells = 1;
  ctx_retain(ctx);
  *out = p;
  return ABX_OK;
}

int abx_particles_destroy(abx_particles *p) {
  particles_release(p);  // freed once no operator refers to it
  return ABX_OK;
}

int abx_particles_set(abx_particles *p, int64_t n, const double *pos, const int64_t *ids) {
  ABX_REQUIRE(p, ABX_ERR_INVALID, "null particles");
  ABX_REQUIRE(n >= 0, ABX_ERR_INVALID, "negative particle count");
  ABX_REQUIRE(n == 0 || pos, ABX_ERR_INVALID, "null positions");
  ABX_TRY(ctx_activate(p->ctx));
  cudaStream_t s = p->ctx->stream;
  const int D = p->dim;
  ABX_TRY(p->pos.reserve((size_t)D * (n ? n : 1)));
  ABX_TRY(p->ids.reserve(n ? n : 1));
  if (n > 0) {
    const void *dpos;
    ABX_TRY(p->stage_a.in(p->ctx, pos, (size_t)n * D * sizeof(double), &dpos));
    k_aos_to_soa<<<ceil_div(n, TPB), TPB, 0, s>>>((const double *)dpos, n, D, p->pos.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    if (ids) {
      const void *dids;
      ABX_TRY(p->stage_b.in(p->ctx, ids, (size_t)n * sizeof(int64_t), &dids));
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->ids.ptr, dids, n * sizeof(int64_t),
                                     cudaMemcpyDeviceToDevice, s));
    } else {
      k_iota64<<<ceil_div(n, TPB), TPB, 0, s>>>(p->ids.ptr, n, 0);
      ABX_CHECK_CUDA(cudaGetLastError());
    }
  }
  p->n = n;
  p->next_id = n;
  p->has_scalar = false;
  p->searchable = false;
  ++p->version;
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

int abx_particles_set_scalar(abx_particles *p, const double *sv) {
  ABX_REQUIRE(p && sv, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  ABX_TRY(p->scalar.reserve(p->n ? p->n : 1));
  if (p->n) {
    const void *d;
    ABX_TRY(p->stage_a.in(p->ctx, sv, p->n * sizeof(double), &d));
    ABX_CHECK_CUDA(cudaMemcpyAsync(p->scalar.ptr, d, p->n * sizeof(double),
                                   cudaMemcpyDeviceToDevice, p->ctx->stream));
    ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  }
  p->has_scalar = true;
  ++p->version;
  return ABX_OK;
}

int64_t abx_particles_size(const abx_particles *p) { return p ? p->n : -1; }

int abx_particles_get_positions(abx_particles *p, double *out) {
  ABX_REQUIRE(p && (out || p->n == 0), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  if (p->n == 0) return ABX_OK;
  void *d;
  const size_t bytes = (size_t)p->n * p->dim * sizeof(double);
  ABX_TRY(p->stage_a.out(p->ctx, out, bytes, &d));
  k_soa_to_aos<<<ceil_div(p->n, TPB), TPB, 0, p->ctx->stream>>>(p->pos.ptr, p->n, p->dim,
                                                                (double *)d);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_TRY(p->stage_a.finish(p->ctx, out, bytes));
  ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return ABX_OK;
}

int abx_particles_get_ids(abx_particles *p, int64_t *out) {
  ABX_REQUIRE(p && (out || p->n == 0), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  if (p->n == 0) return ABX_OK;
  ABX_CHECK_CUDA(cudaMemcpyAsync(out, p->ids.ptr, p->n * sizeof(int64_t), cudaMemcpyDefault,
                                 p->ctx->stream));
  ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return ABX_OK;
}

int abx_particles_get_scalar(abx_particles *p, double *out) {
  ABX_REQUIRE(p && (out || p->n == 0), ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(p->has_scalar, ABX_ERR_STATE, "particle set has no scalar column");
  ABX_TRY(ctx_activate(p->ctx));
  if (p->n == 0) return ABX_OK;
  ABX_CHECK_CUDA(cudaMemcpyAsync(out, p->scalar.ptr, p->n * sizeof(double), cudaMemcpyDefault,
                                 p->ctx->stream));
  ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return ABX_OK;
}

int abx_particles_init_neighbour_search(abx_particles *p, const double *lo, const double *hi,
                                        const int *periodic, double n_leaf) {
  ABX_REQUIRE(p && lo && hi && periodic, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(n_leaf > 0, ABX_ERR_INVALID, "n_particles_in_leaf must be positive");
  for (int d = 0; d < p->dim; ++d)
    ABX_REQUIRE(hi[d] > lo[d], ABX_ERR_INVALID, "empty domain in dimension %d", d);
  ABX_TRY(ctx_activate(p->ctx));
  for (int d = 0; d < p->dim; ++d) {
    p->grid.lo[d] = lo[d];
    p->grid.hi[d] = hi[d];
    p->grid.periodic[d] = periodic[d] ? 1 : 0;
  }
  p->grid.dim = p->dim;
  p->n_leaf = n_leaf;
  p->domain_set = true;
  // neighbour_search_base::set_domain -> set_domain_impl with the current
  // alive count (src/NeighbourSearchBase.h:252-268), then update_positions.
  set_domain_impl(p, (size_t)p->n_alive_prev);
  return update_positions(p);
}

int abx_particles_init_octree(abx_particles *p, const double *lo, const double *hi,
                              const int *periodic, double n_leaf) {
  ABX_REQUIRE(p && lo && hi && periodic, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(n_leaf >= 1, ABX_ERR_INVALID, "n_particles_in_leaf must be >= 1");
  for (int d = 0; d < p->dim; ++d)
    ABX_REQUIRE(hi[d] > lo[d], ABX_ERR_INVALID, "empty domain in dimension %d", d);
  ABX_TRY(ctx_activate(p->ctx));
  for (int d = 0; d < 3; ++d) {
    const bool real = d < p->dim;
    p->grid.lo[d] = real ? lo[d] : 0.0;
    p->grid.hi[d] = real ? hi[d] : 1.0;
    p->grid.periodic[d] = real && periodic[d] ? 1 : 0;
    p->grid.size[d] = 1;
    p->grid.side[d] = real ? hi[d] - lo[d] : 1.0;
    p->grid.inv_side[d] = 1.0 / p->grid.side[d];
  }
  p->grid.dim = p->dim;
  p->grid.ncells = 1;
  p->n_leaf = n_leaf;
  p->domain_set = true;
  p->search_kind = 1;
  return update_positions(p);
}

int abx_particles_get_tree_leaves(abx_particles *p, int64_t *nleaves, int32_t *level,
                                  int32_t *tag, int32_t *begin, int32_t *end, int64_t cap) {
  ABX_REQUIRE(p && nleaves, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(p->searchable && p->search_kind == 1, ABX_ERR_STATE,
              "the particle set has no octree (call abx_particles_init_octree)");
  const OctTree &T = p->tree;
  *nleaves = (int64_t)T.leaves.size();
  if (!level && !tag && !begin && !end) return ABX_OK;
  ABX_REQUIRE(cap >= (int64_t)T.leaves.size(), ABX_ERR_CAPACITY, "leaf capacity too small");
  for (size_t i = 0; i < T.leaves.size(); ++i) {
    const int nd = T.leaves[i];
    if (level) level[i] = T.level[nd];
    if (tag) tag[i] = T.tag[nd];
    if (begin) begin[i] = T.begin[nd];
    if (end) end[i] = T.end[nd];
  }
  return ABX_OK;
}

int abx_particles_set_positions(abx_particles *p, const double *pos) {
  ABX_REQUIRE(p && (pos || p->n == 0), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  if (p->n == 0) return ABX_OK;
  const void *d;
  ABX_TRY(p->stage_a.in(p->ctx, pos, (size_t)p->n * p->dim * sizeof(double), &d));
  k_aos_to_soa<<<ceil_div(p->n, TPB), TPB, 0, p->ctx->stream>>>((const double *)d, p->n, p->dim,
                                                                p->pos.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  p->searchable = false;
  ++p->version;
  return ABX_OK;
}

int abx_particles_update_positions(abx_particles *p) {
  ABX_REQUIRE(p, ABX_ERR_INVALID, "null particles");
  ABX_REQUIRE(p->domain_set, ABX_ERR_STATE, "init_neighbour_search not called");
  ABX_TRY(ctx_activate(p->ctx));
  return update_positions(p);
}

int abx_particles_push_back(abx_particles *p, int64_t n_new, const double *pos, int64_t *ids_out) {
  ABX_REQUIRE(p && (pos || n_new == 0), ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(n_new >= 0, ABX_ERR_INVALID, "negative particle count");
  ABX_TRY(ctx_activate(p->ctx));
  if (n_new == 0) return ABX_OK;
  cudaStream_t s = p->ctx->stream;
  const int D = p->dim;
  const int64_t n0 = p->n, n = n0 + n_new;
  const void *dpos;
  ABX_TRY(p->stage_a.in(p->ctx, pos, (size_t)n_new * D * sizeof(double), &dpos));
  // grow the SoA columns into the alternate buffers, then swap
  ABX_TRY(p->pos_alt.reserve((size_t)D * n));
  ABX_TRY(p->ids_alt.reserve(n));
  for (int d = 0; d < D; ++d)
    if (n0)
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->pos_alt.ptr + (size_t)d * n, p->pos.ptr + (size_t)d * n0,
                                     n0 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  k_append_aos<<<ceil_div(n_new, TPB), TPB, 0, s>>>((const double *)dpos, n_new, D, n0, n,
                                                   p->pos_alt.ptr);
  if (n0)
    ABX_CHECK_CUDA(cudaMemcpyAsync(p->ids_alt.ptr, p->ids.ptr, n0 * sizeof(int64_t),
                                   cudaMemcpyDeviceToDevice, s));
  k_iota64<<<ceil_div(n_new, TPB), TPB, 0, s>>>(p->ids_alt.ptr + n0, n_new, p->next_id);
  ABX_CHECK_CUDA(cudaGetLastError());
  if (p->has_scalar) {
    ABX_TRY(p->scalar_alt.reserve(n));
    if (n0)
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->scalar_alt.ptr, p->scalar.ptr, n0 * sizeof(double),
                                     cudaMemcpyDeviceToDevice, s));
    ABX_CHECK_CUDA(cudaMemsetAsync(p->scalar_alt.ptr + n0, 0, n_new * sizeof(double), s));
    std::swap(p->scalar.ptr, p->scalar_alt.ptr);
    std::swap(p->scalar.cap, p->scalar_alt.cap);
  }
  std::swap(p->pos.ptr, p->pos_alt.ptr);
  std::swap(p->pos.cap, p->pos_alt.cap);
  std::swap(p->ids.ptr, p->ids_alt.ptr);
  std::swap(p->ids.cap, p->ids_alt.cap);
  if (ids_out)
    for (int64_t k = 0; k < n_new; ++k) ids_out[k] = p->next_id + k;
  p->next_id += n_new;
  p->n = n;
  ++p->version;
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  // Particles::push_back on a searchable, ordered set updates the whole
  // search structure (src/Particles.h:264-283)
  if (p->searchable) return update_positions(p);
  return ABX_OK;
}

int abx_particles_erase(abx_particles *p, int64_t first, int64_t last) {
  ABX_REQUIRE(p, ABX_ERR_INVALID, "null particles");
  ABX_REQUIRE(first >= 0 && first <= last && last <= p->n, ABX_ERR_INVALID,
              "erase range [%lld, %lld) outside [0, %lld)", (long long)first, (long long)last,
              (long long)p->n);
  ABX_TRY(ctx_activate(p->ctx));
  if (first == last) return ABX_OK;
  // Particles::erase sets alive = false and updates the search structure,
  // which drops the dead (src/Particles.h:361-389); a non-finite position is
  // dead in the same update
  k_mark_dead<<<ceil_div(last - first, TPB), TPB, 0, p->ctx->stream>>>(p->pos.ptr, first, last);
  ABX_CHECK_CUDA(cudaGetLastError());
  ++p->version;
  if (p->domain_set) return update_positions(p);
  // no search structure yet: compact on the host side of the columns
  const int64_t n = p->n, k = last - first, D = p->dim;
  cudaStream_t s = p->ctx->stream;
  ABX_TRY(p->pos_alt.reserve((size_t)D * (n - k) + 1));
  ABX_TRY(p->ids_alt.reserve(n - k + 1));
  for (int d = 0; d < D; ++d) {
    if (first)
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->pos_alt.ptr + (size_t)d * (n - k), p->pos.ptr + (size_t)d * n,
                                     first * 8, cudaMemcpyDeviceToDevice, s));
    if (n - last)
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->pos_alt.ptr + (size_t)d * (n - k) + first,
                                     p->pos.ptr + (size_t)d * n + last, (n - last) * 8,
                                     cudaMemcpyDeviceToDevice, s));
  }
  if (first)
    ABX_CHECK_CUDA(cudaMemcpyAsync(p->ids_alt.ptr, p->ids.ptr, first * 8, cudaMemcpyDeviceToDevice, s));
  if (n - last)
    ABX_CHECK_CUDA(cudaMemcpyAsync(p->ids_alt.ptr + first, p->ids.ptr + last, (n - last) * 8,
                                   cudaMemcpyDeviceToDevice, s));
  if (p->has_scalar) {
    ABX_TRY(p->scalar_alt.reserve(n - k + 1));
    if (first)
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->scalar_alt.ptr, p->scalar.ptr, first * 8,
                                     cudaMemcpyDeviceToDevice, s));
    if (n - last)
      ABX_CHECK_CUDA(cudaMemcpyAsync(p->scalar_alt.ptr + first, p->scalar.ptr + last,
                                     (n - last) * 8, cudaMemcpyDeviceToDevice, s));
    std::swap(p->scalar.ptr, p->scalar_alt.ptr);
    std::swap(p->scalar.cap, p->scalar_alt.cap);
  }
  std::swap(p->pos.ptr, p->pos_alt.ptr);
  std::swap(p->pos.cap, p->pos_alt.cap);
  std::swap(p->ids.ptr, p->ids_alt.ptr);
  std::swap(p->ids.cap, p->ids_alt.cap);
  p->n = n - k;
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

int abx_particles_find_ids(abx_particles *p, int64_t nq, const int64_t *ids, int64_t *index_out) {
  ABX_REQUIRE(p && ((ids && index_out) || nq == 0), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  if (nq == 0) return ABX_OK;
  cudaStream_t s = p->ctx->stream;
  const int64_t n = p->n;
  ABX_REQUIRE(n < (int64_t)0xFFFFFFFFll, ABX_ERR_INVALID, "too many particles");
  if (p->idmap_version != p->version) {
    // (id, storage index) sorted by id: stable LSD radix sort of the id's
    // two 32-bit halves (low half first), ids as unsigned 64-bit keys
    ABX_TRY(p->idmap_key.reserve(n ? n : 1));
    ABX_TRY(p->idmap_val.reserve(n ? n : 1));
    if (n) {
      size_t off = 0;
      carve_size<uint32_t>(off, n);
      carve_size<uint32_t>(off, n);
      carve_size<uint32_t>(off, n);
      carve_size<uint32_t>(off, n);
      carve_size<uint32_t>(off, n);
      carve_size<uint32_t>(off, radix_temp_u32(n));
      ABX_TRY(p->ctx->scratch.reserve(off + 256));
      unsigned char *base = p->ctx->scratch.ptr;
      off = 0;
      uint32_t *k = carve<uint32_t>(base, off, n);
      uint32_t *v = carve<uint32_t>(base, off, n);
      uint32_t *ka = carve<uint32_t>(base, off, n);
      uint32_t *va = carve<uint32_t>(base, off, n);
      uint32_t *perm = carve<uint32_t>(base, off, n);
      uint32_t *tmp = carve<uint32_t>(base, off, radix_temp_u32(n));
      k_id_half<<<ceil_div(n, TPB), TPB, 0, s>>>(p->ids.ptr, nullptr, n, 0, k, v);
      ABX_TRY(radix_sort_pairs(k, v, n, 32, ka, va, tmp, s));
      k_id_half<<<ceil_div(n, TPB), TPB, 0, s>>>(p->ids.ptr, v, n, 1, k, perm);
      ABX_TRY(radix_sort_pairs(k, perm, n, 32, ka, va, tmp, s));
      k_idmap_fill<<<ceil_div(n, TPB), TPB, 0, s>>>(p->ids.ptr, perm, n, p->idmap_key.ptr,
                                                     p->idmap_val.ptr);
      ABX_CHECK_CUDA(cudaGetLastError());
    }
    p->idmap_version = p->version;
  }
  const void *dq;
  void *dout;
  HostStage out;
  ABX_TRY(p->stage_b.in(p->ctx, ids, nq * sizeof(int64_t), &dq));
  ABX_TRY(out.out(p->ctx, index_out, nq * sizeof(int64_t), &dout));
  k_find_ids<<<ceil_div(nq, TPB), TPB, 0, s>>>(p->idmap_key.ptr, p->idmap_val.ptr, n,
                                               (const int64_t *)dq, nq, (int64_t *)dout);
  ABX_CHECK_CUDA(cudaGetLastError());
  ABX_TRY(out.finish(p->ctx, index_out, nq * sizeof(int64_t)));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

int abx_particles_get_grid(abx_particles *p, uint32_t *size, double *side, uint32_t *ncells) {
  ABX_REQUIRE(p, ABX_ERR_INVALID, "null particles");
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called");
  for (int d = 0; d < p->dim; ++d) {
    if (size) size[d] = p->grid.size[d];
    if (side) side[d] = p->grid.side[d];
  }
  if (ncells) *ncells = p->grid.ncells;
  return ABX_OK;
}

int abx_particles_get_buckets(abx_particles *p, uint32_t *bb, uint32_t *be, uint32_t *keys) {
  ABX_REQUIRE(p, ABX_ERR_INVALID, "null particles");
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called");
  ABX_TRY(ctx_activate(p->ctx));
  cudaStream_t s = p->ctx->stream;
  const size_t nc = p->grid.ncells;
  if (bb) ABX_CHECK_CUDA(cudaMemcpyAsync(bb, p->bucket_begin.ptr, nc * 4, cudaMemcpyDefault, s));
  if (be) ABX_CHECK_CUDA(cudaMemcpyAsync(be, p->bucket_end.ptr, nc * 4, cudaMemcpyDefault, s));
  if (keys && p->n)
    ABX_CHECK_CUDA(cudaMemcpyAsync(keys, p->keys.ptr, p->n * 4, cudaMemcpyDefault, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

int abx_particles_get_view(abx_particles *p, abx_particles_view *out) {
  ABX_REQUIRE(p && out, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called");
  ABX_TRY(ctx_activate(p->ctx));
  ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  std::memset(out, 0, sizeof(*out));
  out->n = p->n;
  out->dim = p->dim;
  out->device = p->ctx->device;
  out->pos = p->pos.ptr;
  out->ids = p->ids.ptr;
  out->search_kind = p->search_kind;
  const bool cells = p->search_kind == 0;
  out->bucket_begin = cells ? p->bucket_begin.ptr : nullptr;
  out->bucket_end = cells ? p->bucket_end.ptr : nullptr;
  out->ncells = cells ? p->grid.ncells : 0;
  for (int d = 0; d < 3; ++d) {
    out->size[d] = p->grid.size[d];
    out->lo[d] = p->grid.lo[d];
    out->hi[d] = p->grid.hi[d];
    out->side[d] = p->grid.side[d];
    out->periodic[d] = p->grid.periodic[d];
  }
  return ABX_OK;
}

}  // extern "C"
