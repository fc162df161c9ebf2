// HyperOctree construction and the FMM's dual-tree traversal on the GPU.
//
// Tree (HyperOctree::build_tree, src/OctTree.h:328-475): level by level, every
// internal node of the previous level gets 2^D child slots in creation order;
// a child's particle range is found by binary search of its tag prefix in
// the sorted tags (point_to_tag, src/detail/SpatialUtil.h:255-286), and it is
// a leaf when it holds at most n_leaf particles or sits on the last level.
// One thread per child slot; the internal children, compacted by a scan,
// are the next level's parents.  The node arrays are then copied to the host
// tree once (the Schwarz domains and the leaf queries read them there).
//
// Traversal (the reference FMM's dual-tree recursion with theta_condition,
// src/FastMultipoleMethod.h:111-548, src/detail/FastMultipoleMethod.h:
// 1249-1279): level by level, each target node takes its parent's near list;
// a near leaf stays near, a near internal node is replaced by its non-empty
// children, each of which is near (admissibility fails) or an M2L source.
// Leaves then take every leaf under their near list as P2P sources.  Count
// and fill passes with scans make every list a CSR array; the M2L pairs are
// keyed by (level, integer box offset) and grouped by that key with a stable
// radix sort for the tensor-core M2L.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "handles.cuh"

namespace abx {
namespace {

constexpr int OT_TPB = 256;

__device__ __forceinline__ int lower_bound_u32(const uint32_t *a, int lo, int hi, uint32_t v) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int upper_bound_u32(const uint32_t *a, int lo, int hi, uint32_t v) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

struct NodeArrays {
  int *tag, *level, *begin, *end, *kind, *first_child, *parent;
};

__global__ void k_oct_children(const uint32_t *__restrict__ tags, const int *__restrict__ active,
                               int nactive, int nch, int base, int level, int shift,
                               uint32_t length, double n_leaf, int max_level, NodeArrays N,
                               uint32_t *__restrict__ internal) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nactive * nch) return;
  const int k = j / nch, c = j - k * nch;
  const int a = active[k];
  const uint32_t mask = (uint32_t)N.tag[a] | ((uint32_t)c << shift);
  const int lb = lower_bound_u32(tags, N.begin[a], N.end[a], mask);
  const int ub = upper_bound_u32(tags, lb, N.end[a], mask + length);
  const int id = base + j;
  const int count = ub - lb;
  int kind = 0;
  if (count > 0) kind = (level == max_level || (double)count <= n_leaf) ? 1 : 2;
  N.tag[id] = (int)mask;
  N.level[id] = level;
  N.begin[id] = lb;
  N.end[id] = ub;
  N.kind[id] = kind;
  N.first_child[id] = -1;
  N.parent[id] = a;
  internal[j] = kind == 2 ? 1u : 0u;
  if (c == 0) N.first_child[a] = base + k * nch;
}

__global__ void k_compact_ids(const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos,
                              int n, int base, int *__restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n && flag[j]) out[pos[j]] = base + j;
}

__global__ void k_flag_kind(const int *__restrict__ kind, int n, int want,
                            uint32_t *__restrict__ flag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) flag[j] = kind[j] == want ? 1u : 0u;
}

// Exclusive scan of n u32 flags/counts in place; returns the total.
int scan_total(uint32_t *v, int n, DevBuf<uint32_t> &tmp, cudaStream_t s, uint32_t *total) {
  if (n == 0) {
    *total = 0;
    return ABX_OK;
  }
  uint32_t last = 0;
  ABX_CHECK_CUDA(cudaMemcpyAsync(&last, v + n - 1, 4, cudaMemcpyDeviceToHost, s));
  ABX_TRY(tmp.reserve(scan_temp_elems(n) + 64));
  ABX_TRY(exclusive_scan_u32(v, n, tmp.ptr, s));
  uint32_t lastx = 0;
  ABX_CHECK_CUDA(cudaMemcpyAsync(&lastx, v + n - 1, 4, cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  *total = last + lastx;
  return ABX_OK;
}

// grow every node array to hold `need` nodes, keeping the first `keep`
int grow_nodes(OctDev &T, int need, int keep, cudaStream_t s) {
  if (need <= T.cap) return ABX_OK;
  const int cap = std::max(need, 2 * T.cap);
  DevBuf<int> *arrs[7] = {&T.tag, &T.level, &T.begin, &T.end, &T.kind, &T.first_child, &T.parent};
  for (DevBuf<int> *a : arrs) {
    DevBuf<int> nb;
    ABX_TRY(nb.reserve(cap));
    if (keep)
      ABX_CHECK_CUDA(cudaMemcpyAsync(nb.ptr, a->ptr, (size_t)keep * 4, cudaMemcpyDeviceToDevice, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    std::swap(a->ptr, nb.ptr);
    std::swap(a->cap, nb.cap);
  }
  T.cap = cap;
  return ABX_OK;
}

NodeArrays node_arrays(OctDev &T) {
  return NodeArrays{T.tag.ptr, T.level.ptr, T.begin.ptr, T.end.ptr, T.kind.ptr, T.first_child.ptr,
                    T.parent.ptr};
}

// ----------------------------------------------------------- traversal ---
struct BoxView {
  const double *box;  // nnodes x 6: lo[3], hi[3]
  int D;
};

// The reference's admissibility test scaled by eta (eta = 1:
// theta_condition): near iff max_diam^2 > eta^2 dist^2, dist the box gap.
__device__ __forceinline__ bool near_pair(const BoxView &B, int t, int s, double eta2) {
  const double *bt = B.box + (size_t)t * 6, *bs = B.box + (size_t)s * 6;
  double maxd = 2.2250738585072014e-308;  // numeric_limits<double>::min()
  for (int d = 0; d < B.D; ++d) maxd = fmax(maxd, __dsub_rn(bt[3 + d], bt[d]));
  double dist2 = 0.0;
  for (int d = 0; d < B.D; ++d) {
    double dd = 0.0;
    const double tlo = bt[d], thi = bt[3 + d], slo = bs[d], shi = bs[3 + d];
    if (thi < slo) dd = __dsub_rn(slo, thi);
    else if (shi < tlo) dd = __dsub_rn(tlo, shi);
    maxd = fmax(maxd, __dsub_rn(shi, slo));
    dist2 = __dadd_rn(dist2, __dmul_rn(dd, dd));
  }
  return __dmul_rn(maxd, maxd) > __dmul_rn(eta2, dist2);
}

// Per target node t of a level: from the parent's near list, count (FILL =
// false) or write (FILL = true) t's near list and its M2L sources.
template <bool FILL>
__global__ void k_trav_level(int base, int count, int pbase, const int *__restrict__ prp,
                             const int *__restrict__ pidx, const int *__restrict__ kind,
                             const int *__restrict__ first_child, const int *__restrict__ parent,
                             int nch, BoxView B, double eta2, uint32_t *__restrict__ ncnt,
                             uint32_t *__restrict__ mcnt, const uint32_t *__restrict__ noff,
                             const uint32_t *__restrict__ moff, int *__restrict__ nidx,
                             int2 *__restrict__ mpairs, int64_t mbase) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const int t = base + j;
  uint32_t nc = 0, mc = 0;
  if (kind[t] != 0) {
    const int pa = parent[t] - pbase;
    for (int q = prp[pa]; q < prp[pa + 1]; ++q) {
      const int sdx = pidx[q];
      if (kind[sdx] == 1) {
        if (FILL) nidx[noff[j] + nc] = sdx;
        ++nc;
        continue;
      }
      const int fc = first_child[sdx];
      for (int c = 0; c < nch; ++c) {
        const int ch = fc + c;
        if (kind[ch] == 0) continue;
        if (near_pair(B, t, ch, eta2)) {
          if (FILL) nidx[noff[j] + nc] = ch;
          ++nc;
        } else {
          if (FILL) mpairs[mbase + moff[j] + mc] = make_int2(t, ch);
          ++mc;
        }
      }
    }
  }
  if (!FILL) {
    ncnt[j] = nc;
    mcnt[j] = mc;
  }
}

// P2P sources of the leaves of one level: every leaf under the near list
// (a near leaf itself, or the leaves of a near internal node: those whose
// particle range starts inside the node's, a contiguous run of the leaves
// sorted by their first particle).
template <bool FILL>
__global__ void k_p2p_level(int base, int count, const int *__restrict__ rp,
                            const int *__restrict__ idx, const int *__restrict__ kind,
                            const int *__restrict__ nbegin, const int *__restrict__ nend,
                            const int *__restrict__ leaf_of_node, const int *__restrict__ lb_begin,
                            const int *__restrict__ lb_node, int nleaves,
                            uint32_t *__restrict__ cnt, const uint32_t *__restrict__ off,
                            int *__restrict__ src) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const int t = base + j;
  if (kind[t] != 1) return;
  const int row = leaf_of_node[t];
  uint32_t c = 0;
  for (int q = rp[j]; q < rp[j + 1]; ++q) {
    const int sdx = idx[q];
    if (kind[sdx] == 1) {
      if (FILL) src[off[row] + c] = sdx;
      ++c;
      continue;
    }
    // leaves with first particle in [begin, end) of sdx
    int lo = 0, hi = nleaves;
    const int b0 = nbegin[sdx], b1 = nend[sdx];
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (lb_begin[mid] < b0) lo = mid + 1; else hi = mid;
    }
    for (int k = lo; k < nleaves && lb_begin[k] < b1; ++k) {
      if (FILL) src[off[row] + c] = lb_node[k];
      ++c;
    }
  }
  if (!FILL) cnt[row] = c;
}

__global__ void k_leaf_rows(const int *__restrict__ leaves, int nleaves,
                            int *__restrict__ leaf_of_node) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nleaves) leaf_of_node[leaves[k]] = k;
}

// integer box coordinate of a node along dimension d (its tag's bits)
__device__ __forceinline__ int box_coord(int tag, int level, int max_level, int D, int d) {
  int c = 0;
  for (int l = 1; l <= level; ++l) c = (c << 1) | ((tag >> ((max_level - l) * D + (D - 1 - d))) & 1);
  return c;
}

// M2L matrix key (level, box offset) of every pair as a dense code; with
// code == null only the largest offset is measured.
__global__ void k_m2l_codes(const int2 *__restrict__ pairs, int64_t npairs,
                            const int *__restrict__ tag, const int *__restrict__ level,
                            int max_level, int D, int R, uint32_t *__restrict__ code,
                            uint32_t *__restrict__ used, unsigned int *__restrict__ rmax) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npairs) return;
  const int2 pr = pairs[q];
  const int L = level[pr.x];
  const int W = 2 * R + 1;
  uint32_t cd = (uint32_t)L;
  unsigned int m = 0;
  for (int d = 0; d < 3; ++d) {
    int o = 0;
    if (d < D)
      o = box_coord(tag[pr.y], L, max_level, D, d) - box_coord(tag[pr.x], L, max_level, D, d);
    m = max(m, (unsigned int)abs(o));
    cd = cd * (uint32_t)W + (uint32_t)(min(max(o, -R), R) + R);
  }
  if (rmax) atomicMax(rmax, m);
  if (code) {
    code[q] = cd;
    used[cd] = 1u;
  }
}

__global__ void k_code_to_mat(const uint32_t *__restrict__ code, int64_t npairs,
                              const uint32_t *__restrict__ matid_of_code,
                              uint32_t *__restrict__ mat, uint32_t *__restrict__ iota) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npairs) return;
  mat[q] = matid_of_code[code[q]];
  iota[q] = (uint32_t)q;
}

__global__ void k_group_pairs(const int2 *__restrict__ pairs, const uint32_t *__restrict__ mat,
                              const uint32_t *__restrict__ order, int64_t npairs,
                              int2 *__restrict__ bymat, int *__restrict__ trip,
                              uint32_t *__restrict__ mat_count) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npairs) return;
  const int2 pr = pairs[order[k]];
  const uint32_t m = mat[k];
  bymat[k] = pr;
  trip[3 * k] = pr.x;
  trip[3 * k + 1] = pr.y;
  trip[3 * k + 2] = (int)m;
  atomicAdd(&mat_count[m], 1u);
}

// the first pair's target of every matrix (a representative for its box size)
__global__ void k_mat_rep(const int2 *__restrict__ bymat, const int *__restrict__ mat_off,
                          int nmat, int *__restrict__ rep) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < nmat) rep[m] = bymat[mat_off[m]].x;
}

}  // namespace

// HyperOctree::build_tree on the device from the sorted tags of the na > 0
// alive particles; fills p->oct (device) and p->tree (host copy).
int octree_build_device(abx_particles *p, const uint32_t *tags, int64_t na) {
  cudaStream_t s = p->ctx->stream;
  const int D = p->dim, nch = 1 << D;
  OctDev &T = p->oct;
  T.reset();
  T.max_level = 32 / D - 2;
  ABX_REQUIRE(na < (int64_t)0x7fffffff, ABX_ERR_INVALID, "too many particles for the octree");
  ABX_TRY(grow_nodes(T, 1 + nch * 64, 0, s));
  const int root_end = (int)na;
  const int zero = 0, two = 2, minus1 = -1;
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.tag.ptr, &zero, 4, cudaMemcpyHostToDevice, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.level.ptr, &zero, 4, cudaMemcpyHostToDevice, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.begin.ptr, &zero, 4, cudaMemcpyHostToDevice, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.end.ptr, &root_end, 4, cudaMemcpyHostToDevice, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.kind.ptr, &two, 4, cudaMemcpyHostToDevice, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.first_child.ptr, &minus1, 4, cudaMemcpyHostToDevice, s));
  ABX_CHECK_CUDA(cudaMemcpyAsync(T.parent.ptr, &minus1, 4, cudaMemcpyHostToDevice, s));
  T.lvl_base.assign(1, 0);
  T.lvl_count.assign(1, 1);
  DevBuf<int> active, next;
  DevBuf<uint32_t> flag, pos, tmp;
  ABX_TRY(active.reserve(1));
  ABX_CHECK_CUDA(cudaMemcpyAsync(active.ptr, &zero, 4, cudaMemcpyHostToDevice, s));
  int nactive = 1, nn = 1;
  for (int level = 1; nactive > 0; ++level) {
    const int shift = (T.max_level - level) * D;
    const uint32_t length = (uint32_t)((1u << shift) - 1u);
    const int slots = nactive * nch;
    ABX_TRY(grow_nodes(T, nn + slots, nn, s));
    ABX_TRY(flag.reserve(slots + 1));
    ABX_TRY(pos.reserve(slots + 1));
    k_oct_children<<<ceil_div(slots, OT_TPB), OT_TPB, 0, s>>>(
        tags, active.ptr, nactive, nch, nn, level, shift, length, p->n_leaf, T.max_level,
        node_arrays(T), flag.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    // the positions of the internal children among the slots
    ABX_CHECK_CUDA(cudaMemcpyAsync(pos.ptr, flag.ptr, (size_t)slots * 4, cudaMemcpyDeviceToDevice, s));
    uint32_t ninternal = 0;
    ABX_TRY(scan_total(pos.ptr, slots, tmp, s, &ninternal));
    ABX_TRY(next.reserve(ninternal ? ninternal : 1));
    k_compact_ids<<<ceil_div(slots, OT_TPB), OT_TPB, 0, s>>>(flag.ptr, pos.ptr, slots, nn, next.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    T.lvl_base.push_back(nn);
    T.lvl_count.push_back(slots);
    nn += slots;
    nactive = (int)ninternal;
    std::swap(active.ptr, next.ptr);
    std::swap(active.cap, next.cap);
  }
  T.nnodes = nn;
  // leaves in creation (node id) order
  ABX_TRY(flag.reserve(nn + 1));
  ABX_TRY(pos.reserve(nn + 1));
  k_flag_kind<<<ceil_div(nn, OT_TPB), OT_TPB, 0, s>>>(T.kind.ptr, nn, 1, flag.ptr);
  ABX_CHECK_CUDA(cudaMemcpyAsync(pos.ptr, flag.ptr, (size_t)nn * 4, cudaMemcpyDeviceToDevice, s));
  uint32_t nl = 0;
  ABX_TRY(scan_total(pos.ptr, nn, tmp, s, &nl));
  ABX_TRY(T.leaves.reserve(nl ? nl : 1));
  k_compact_ids<<<ceil_div(nn, OT_TPB), OT_TPB, 0, s>>>(flag.ptr, pos.ptr, nn, 0, T.leaves.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  T.nleaves = (int)nl;
  // the host copy
  OctTree &H = p->tree;
  H = OctTree();
  H.dim = D;
  H.max_level = T.max_level;
  std::vector<int> *hv[7] = {&H.tag, &H.level, &H.begin, &H.end, &H.kind, &H.first_child, &H.parent};
  DevBuf<int> *dv[7] = {&T.tag, &T.level, &T.begin, &T.end, &T.kind, &T.first_child, &T.parent};
  for (int a = 0; a < 7; ++a) {
    hv[a]->resize(nn);
    ABX_CHECK_CUDA(cudaMemcpyAsync(hv[a]->data(), dv[a]->ptr, (size_t)nn * 4, cudaMemcpyDeviceToHost, s));
  }
  H.leaves.resize(nl);
  if (nl)
    ABX_CHECK_CUDA(cudaMemcpyAsync(H.leaves.data(), T.leaves.ptr, (size_t)nl * 4,
                                   cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

// The FMM plan's lists from the device tree: M2L pairs grouped by matrix key,
// the near-field P2P lists of the leaves.  boxes: nnodes x 6 on the device.
int fmm_traverse_device(abx_particles *p, const double *boxes, double eta, FmmLists &out) {
  cudaStream_t s = p->ctx->stream;
  OctDev &T = p->oct;
  const int D = p->dim, nch = 1 << D;
  const BoxView B{boxes, D};
  const double eta2 = eta * eta;
  const int nlev = (int)T.lvl_base.size();
  DevBuf<uint32_t> tmp;
  // per level: near lists (CSR over the level's nodes); level 0 is the root
  // with itself as its near list
  std::vector<DevBuf<int>> lrp(nlev), lidx(nlev);
  ABX_TRY(lrp[0].reserve(2));
  ABX_TRY(lidx[0].reserve(1));
  {
    const int h[2] = {0, 1}, zero = 0;
    ABX_CHECK_CUDA(cudaMemcpyAsync(lrp[0].ptr, h, 8, cudaMemcpyHostToDevice, s));
    ABX_CHECK_CUDA(cudaMemcpyAsync(lidx[0].ptr, &zero, 4, cudaMemcpyHostToDevice, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  DevBuf<int2> mpairs;
  int64_t nm2l = 0;
  DevBuf<uint32_t> ncnt, mcnt;
  for (int L = 1; L < nlev; ++L) {
    const int base = T.lvl_base[L], count = T.lvl_count[L], pbase = T.lvl_base[L - 1];
    ABX_TRY(ncnt.reserve(count + 1));
    ABX_TRY(mcnt.reserve(count + 1));
    k_trav_level<false><<<ceil_div(count, OT_TPB), OT_TPB, 0, s>>>(
        base, count, pbase, lrp[L - 1].ptr, lidx[L - 1].ptr, T.kind.ptr, T.first_child.ptr,
        T.parent.ptr, nch, B, eta2, ncnt.ptr, mcnt.ptr, nullptr, nullptr, nullptr, nullptr, 0);
    ABX_CHECK_CUDA(cudaGetLastError());
    uint32_t ntot = 0, mtot = 0;
    ABX_TRY(scan_total(ncnt.ptr, count, tmp, s, &ntot));
    ABX_TRY(scan_total(mcnt.ptr, count, tmp, s, &mtot));
    // rowptr = the scanned counts, then the total
    ABX_TRY(lrp[L].reserve(count + 1));
    ABX_CHECK_CUDA(cudaMemcpyAsync(lrp[L].ptr, ncnt.ptr, (size_t)count * 4, cudaMemcpyDeviceToDevice, s));
    const int ntot_i = (int)ntot;
    ABX_CHECK_CUDA(cudaMemcpyAsync(lrp[L].ptr + count, &ntot_i, 4, cudaMemcpyHostToDevice, s));
    ABX_TRY(lidx[L].reserve(ntot ? ntot : 1));
    if (mtot) {
      DevBuf<int2> grown;
      ABX_TRY(grown.reserve((size_t)nm2l + mtot));
      if (nm2l)
        ABX_CHECK_CUDA(cudaMemcpyAsync(grown.ptr, mpairs.ptr, (size_t)nm2l * sizeof(int2),
                                       cudaMemcpyDeviceToDevice, s));
      ABX_CHECK_CUDA(cudaStreamSynchronize(s));
      std::swap(grown.ptr, mpairs.ptr);
      std::swap(grown.cap, mpairs.cap);
    }
    k_trav_level<true><<<ceil_div(count, OT_TPB), OT_TPB, 0, s>>>(
        base, count, pbase, lrp[L - 1].ptr, lidx[L - 1].ptr, T.kind.ptr, T.first_child.ptr,
        T.parent.ptr, nch, B, eta2, nullptr, nullptr, ncnt.ptr, mcnt.ptr, lidx[L].ptr,
        mpairs.ptr, nm2l);
    ABX_CHECK_CUDA(cudaGetLastError());
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    nm2l += mtot;
  }
  // ---- P2P lists over the leaves (creation order)
  const int nl = T.nleaves, nn = T.nnodes;
  DevBuf<int> leaf_of_node, lb_begin, lb_node;
  ABX_TRY(leaf_of_node.reserve(nn));
  ABX_TRY(lb_begin.reserve(nl ? nl : 1));
  ABX_TRY(lb_node.reserve(nl ? nl : 1));
  std::vector<int> hb(nl), hn(nl);
  {
    const OctTree &H = p->tree;
    std::vector<std::pair<int, int>> bl(nl);
    for (int k = 0; k < nl; ++k) bl[k] = {H.begin[H.leaves[k]], H.leaves[k]};
    std::sort(bl.begin(), bl.end());
    for (int k = 0; k < nl; ++k) {
      hb[k] = bl[k].first;
      hn[k] = bl[k].second;
    }
  }
  if (nl) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(lb_begin.ptr, hb.data(), (size_t)nl * 4, cudaMemcpyHostToDevice, s));
    ABX_CHECK_CUDA(cudaMemcpyAsync(lb_node.ptr, hn.data(), (size_t)nl * 4, cudaMemcpyHostToDevice, s));
    k_leaf_rows<<<ceil_div(nl, OT_TPB), OT_TPB, 0, s>>>(T.leaves.ptr, nl, leaf_of_node.ptr);
  }
  ABX_TRY(out.p2p_rowptr.reserve(nl + 1));
  DevBuf<uint32_t> pcnt;
  ABX_TRY(pcnt.reserve(nl + 1));
  for (int L = 1; L < nlev; ++L)
    k_p2p_level<false><<<ceil_div(T.lvl_count[L], OT_TPB), OT_TPB, 0, s>>>(
        T.lvl_base[L], T.lvl_count[L], lrp[L].ptr, lidx[L].ptr, T.kind.ptr, T.begin.ptr,
        T.end.ptr, leaf_of_node.ptr, lb_begin.ptr, lb_node.ptr, nl, pcnt.ptr, nullptr, nullptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  uint32_t ptot = 0;
  ABX_TRY(scan_total(pcnt.ptr, nl, tmp, s, &ptot));
  ABX_CHECK_CUDA(cudaMemcpyAsync(out.p2p_rowptr.ptr, pcnt.ptr, (size_t)nl * 4, cudaMemcpyDeviceToDevice, s));
  const int ptot_i = (int)ptot;
  ABX_CHECK_CUDA(cudaMemcpyAsync(out.p2p_rowptr.ptr + nl, &ptot_i, 4, cudaMemcpyHostToDevice, s));
  ABX_TRY(out.p2p_src.reserve(ptot ? ptot : 1));
  for (int L = 1; L < nlev; ++L)
    k_p2p_level<true><<<ceil_div(T.lvl_count[L], OT_TPB), OT_TPB, 0, s>>>(
        T.lvl_base[L], T.lvl_count[L], lrp[L].ptr, lidx[L].ptr, T.kind.ptr, T.begin.ptr,
        T.end.ptr, leaf_of_node.ptr, lb_begin.ptr, lb_node.ptr, nl, nullptr, pcnt.ptr,
        out.p2p_src.ptr);
  ABX_CHECK_CUDA(cudaGetLastError());
  // ---- M2L pairs grouped by (level, box offset)
  out.n_m2l = nm2l;
  out.mat_off.assign(1, 0);
  out.mat_rep.clear();
  out.mat_key.clear();
  if (nm2l > 0) {
    DevBuf<unsigned int> rmax;
    ABX_TRY(rmax.reserve(1));
    ABX_CHECK_CUDA(cudaMemsetAsync(rmax.ptr, 0, 4, s));
    k_m2l_codes<<<ceil_div(nm2l, OT_TPB), OT_TPB, 0, s>>>(mpairs.ptr, nm2l, T.tag.ptr, T.level.ptr,
                                                         T.max_level, D, 0, nullptr, nullptr,
                                                         rmax.ptr);
    unsigned int R = 0;
    ABX_CHECK_CUDA(cudaMemcpyAsync(&R, rmax.ptr, 4, cudaMemcpyDeviceToHost, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    const int W = 2 * (int)R + 1;
    const int64_t ncodes = (int64_t)nlev * W * W * W;
    ABX_REQUIRE(ncodes < ((int64_t)1 << 30), ABX_ERR_INVALID, "M2L offsets too spread (%u)", R);
    DevBuf<uint32_t> code, used, mat, iota, mat_alt, iota_alt, rtmp, cnt;
    ABX_TRY(code.reserve(nm2l));
    ABX_TRY(used.reserve(ncodes + 1));
    ABX_CHECK_CUDA(cudaMemsetAsync(used.ptr, 0, (size_t)(ncodes + 1) * 4, s));
    k_m2l_codes<<<ceil_div(nm2l, OT_TPB), OT_TPB, 0, s>>>(mpairs.ptr, nm2l, T.tag.ptr, T.level.ptr,
                                                         T.max_level, D, (int)R, code.ptr,
                                                         used.ptr, nullptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    // matrix ids in increasing key order; the keys themselves for the host
    std::vector<uint32_t> hused(ncodes);
    ABX_CHECK_CUDA(cudaMemcpyAsync(hused.data(), used.ptr, (size_t)ncodes * 4, cudaMemcpyDeviceToHost, s));
    uint32_t nmat = 0;
    ABX_TRY(scan_total(used.ptr, (int)ncodes, tmp, s, &nmat));
    for (int64_t c = 0; c < ncodes; ++c)
      if (hused[c]) {
        int64_t r = c;
        std::array<int, 4> key{0, 0, 0, 0};
        for (int d = 2; d >= 0; --d) {
          key[1 + d] = (int)(r % W) - (int)R;
          r /= W;
        }
        key[0] = (int)r;
        out.mat_key.push_back(key);
      }
    ABX_TRY(mat.reserve(nm2l));
    ABX_TRY(iota.reserve(nm2l));
    ABX_TRY(mat_alt.reserve(nm2l));
    ABX_TRY(iota_alt.reserve(nm2l));
    ABX_TRY(rtmp.reserve(radix_temp_u32(nm2l)));
    k_code_to_mat<<<ceil_div(nm2l, OT_TPB), OT_TPB, 0, s>>>(code.ptr, nm2l, used.ptr, mat.ptr,
                                                           iota.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    int bits = 0;
    while (bits < 32 && ((nmat - 1) >> bits) != 0) ++bits;
    ABX_TRY(radix_sort_pairs(mat.ptr, iota.ptr, nm2l, bits, mat_alt.ptr, iota_alt.ptr, rtmp.ptr, s));
    ABX_TRY(out.m2l_by_mat.reserve(nm2l));
    ABX_TRY(out.m2l_trip.reserve(3 * nm2l));
    ABX_TRY(cnt.reserve(nmat + 1));
    ABX_CHECK_CUDA(cudaMemsetAsync(cnt.ptr, 0, (size_t)(nmat + 1) * 4, s));
    k_group_pairs<<<ceil_div(nm2l, OT_TPB), OT_TPB, 0, s>>>(mpairs.ptr, mat.ptr, iota.ptr, nm2l,
                                                           out.m2l_by_mat.ptr, out.m2l_trip.ptr,
                                                           cnt.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    std::vector<uint32_t> hc(nmat);
    ABX_CHECK_CUDA(cudaMemcpyAsync(hc.data(), cnt.ptr, (size_t)nmat * 4, cudaMemcpyDeviceToHost, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    out.mat_off.assign(nmat + 1, 0);
    for (uint32_t m = 0; m < nmat; ++m) out.mat_off[m + 1] = out.mat_off[m] + (int)hc[m];
    DevBuf<int> moff_d, rep_d;
    ABX_TRY(moff_d.reserve(nmat + 1));
    ABX_TRY(rep_d.reserve(nmat + 1));
    ABX_CHECK_CUDA(cudaMemcpyAsync(moff_d.ptr, out.mat_off.data(), (size_t)(nmat + 1) * 4,
                                   cudaMemcpyHostToDevice, s));
    k_mat_rep<<<ceil_div(nmat, OT_TPB), OT_TPB, 0, s>>>(out.m2l_by_mat.ptr, moff_d.ptr, (int)nmat,
                                                       rep_d.ptr);
    ABX_CHECK_CUDA(cudaGetLastError());
    out.mat_rep.resize(nmat);
    ABX_CHECK_CUDA(cudaMemcpyAsync(out.mat_rep.data(), rep_d.ptr, (size_t)nmat * 4,
                                   cudaMemcpyDeviceToHost, s));
  }
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  return ABX_OK;
}

}  // namespace abx
