// Handle types behind the C ABI: particle sets with their cell list, and
// operators with their pair layout.
#pragma once

#include <array>

#include "common.cuh"

namespace abx {

// Grow-only staging for one vector argument that may be host memory.
struct HostStage {
  DevBuf<unsigned char> buf;
  bool host_ = false;
  int in(abx_context *ctx, const void *user, size_t bytes, const void **dev);
  int out(abx_context *ctx, void *user, size_t bytes, void **dev);
  int finish(abx_context *ctx, void *user, size_t bytes);
};

// The CellListOrdered grid (src/CellListOrdered.h:132-186), padded to 3
// dimensions: unused dimensions have size 1, side 1, and coordinate 0.
struct GridDesc {
  int dim;
  double lo[3], hi[3];
  int periodic[3];
  uint32_t size[3];
  double side[3];
  double inv_side[3];
  uint32_t ncells;
};

// HyperOctree (src/OctTree.h:328-475), kept on the host in the reference's
// layout: nodes level by level, every internal node owning 2^D consecutive
// child slots (empty children included); leaves in the order they are
// created.  Particle ranges index the tag-sorted storage order.
struct OctTree {
  int max_level = 0;
  int dim = 3;
  std::vector<int> tag, level, begin, end, kind, first_child, parent;  // per node
  std::vector<int> leaves;                                              // node ids
  // geometric box of a node (bisection as in point_to_tag)
  void box(const GridDesc &g, int node, double *lo, double *hi) const;
};

// The octree's node arrays on the device (octree.cu), levels as node-id
// ranges: level L holds nodes [lvl_base[L], lvl_base[L] + lvl_count[L]).
struct OctDev {
  DevBuf<int> tag, level, begin, end, kind, first_child, parent, leaves;
  int cap = 0, nnodes = 0, nleaves = 0, max_level = 0;
  std::vector<int> lvl_base, lvl_count;
  void reset() {
    DevBuf<int> *a[8] = {&tag, &level, &begin, &end, &kind, &first_child, &parent, &leaves};
    for (DevBuf<int> *b : a) b->release();
    cap = nnodes = nleaves = max_level = 0;
    lvl_base.clear();
    lvl_count.clear();
  }
};

// The FMM plan's lists built on the device (octree.cu): M2L pairs grouped by
// matrix key (level, integer box offset), and the leaves' P2P sources.
struct FmmLists {
  DevBuf<int2> m2l_by_mat;          // (target, source), grouped by matrix
  DevBuf<int> m2l_trip;             // (target, source, matrix) in the same order
  DevBuf<int> p2p_rowptr, p2p_src;  // CSR over the leaves (creation order)
  std::vector<int> mat_off;         // nmat + 1
  std::vector<std::array<int, 4>> mat_key;  // level, offset (in boxes) per dimension
  std::vector<int> mat_rep;         // a target node of each matrix
  int64_t n_m2l = 0;
};

}  // namespace abx

struct abx_particles {
  std::atomic<int> refs{1};
  abx_context *ctx = nullptr;
  int dim = 3;
  int64_t n = 0;
  // Storage in the current order; positions are SoA: pos[d*n + i].
  abx::DevBuf<double> pos, pos_alt;
  abx::DevBuf<int64_t> ids, ids_alt;
  abx::DevBuf<double> scalar, scalar_alt;
  bool has_scalar = false;
  int64_t next_id = 0;
  // Neighbour search state.
  bool domain_set = false;
  bool searchable = false;
  abx::GridDesc grid{};
  double n_leaf = 10.0;
  size_t size_calculated_with_n = (size_t)-1;  // CellListOrdered.h:106
  int64_t n_alive_prev = 0;                     // m_alive_indices.size()
  abx::DevBuf<uint32_t> keys;                   // sorted bucket key per particle
  abx::DevBuf<uint32_t> bucket_begin, bucket_end;
  int search_kind = 0;  // 0: CellListOrdered, 1: HyperOctree
  abx::OctTree tree;
  uint64_t version = 0;  // bumped by every rebuild; operators check it
  abx::HostStage stage_a, stage_b;
  // cell-list build (celllist.cu): per-dimension cell boundaries of the
  // grid they were computed for, look-back status words, pass epoch
  abx::DevBuf<uint64_t> cl_bnd;
  size_t cl_bnd_off[3] = {0, 0, 0};
  abx::GridDesc cl_bnd_grid{};
  bool cl_bnd_valid = false;
  abx::DevBuf<unsigned long long> cl_status;
  uint32_t cl_epoch = 0;
  // find-by-id map (NeighbourSearchBase::find_id_map): ids sorted, with the
  // storage index of each; rebuilt when the storage version moved
  abx::OctDev oct;  // the octree on the device (search_kind 1)
  abx::DevBuf<int64_t> idmap_key;
  abx::DevBuf<uint32_t> idmap_val;
  uint64_t idmap_version = ~uint64_t(0);
};

namespace abx {
struct PairLayout;   // pairs.cu
struct FmmPlan;      // fmm.cu
}  // namespace abx

struct abx_operator {
  int kind = 0;  // 0 sparse, 1 dense, 2 black-box FMM
  abx_particles *rows = nullptr, *cols = nullptr;
  uint64_t rows_version = 0, cols_version = 0;
  double radius = 0.0;
  abx_kernel k{};
  int precision = ABX_PREC_FP64;
  abx::PairLayout *pairs = nullptr;
  abx::FmmPlan *fmm = nullptr;
  abx::HostStage stage_b, stage_c;
  abx::DevBuf<double> partial;  // dense mixed matvec: row sums per column chunk
  int64_t last_candidates = 0, last_pairs = 0;
};

namespace abx {
struct Schwarz;  // solver.cu
struct Spai;     // spai.cu
}  // namespace abx

// A preconditioner x = M b (restricted additive Schwarz or a sparse
// approximate inverse), applied by abx_gmres_solve.
struct abx_precond {
  int kind = 0;  // 1 Schwarz, 2 sparse approximate inverse
  abx::Schwarz *schwarz = nullptr;
  abx::Spai *spai = nullptr;
  abx_context *ctx = nullptr;
  int64_t n = 0;
  int64_t exact_rows = 0;  // learned approximate inverse: rows solved exactly
  double setup_s = 0.0;    // approximate inverses: set-up time
  // learned approximate inverse: device time of the set-up phases (k-NN,
  // features, inference, exact rows), from CUDA events on the build stream
  double phase_s[4] = {0.0, 0.0, 0.0, 0.0};
  abx::HostStage stage_b, stage_x;
};

namespace abx {
void particles_retain(abx_particles *p);
void particles_release(abx_particles *p);
int particles_grid_desc(const abx_particles *p, GridDesc *g);
// celllist.cu: the CellListOrdered build of the alive particles (n > 0)
int celllist_build(abx_particles *p);
// octree.cu: the HyperOctree from the sorted tags (device and host copies),
// and the FMM traversal lists
int octree_build_device(abx_particles *p, const uint32_t *tags, int64_t na);
int fmm_traverse_device(abx_particles *p, const double *boxes, double eta, FmmLists &out);
// pairs.cu
int pair_layout_build(abx_operator *op);
void pair_layout_free(PairLayout *L);
int sparse_matvec_device(abx_operator *op, const double *b, double *c);
// operators.cu
int dense_matvec_device(abx_operator *op, const double *b, double *c);
// fmm.cu
int fmm_matvec_device(abx_operator *op, const double *b, double *c);
void fmm_plan_free(FmmPlan *P);
}  // namespace abx
