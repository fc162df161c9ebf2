// Oracle for the particle hot path: TEST INFRASTRUCTURE ONLY.
//
// A plain C++17 + OpenMP restatement of the reference algorithms (Aboria,
// header-only C++14).  It is loaded by the test-suite and by the CPU-baseline
// leg of bench.py, and nothing in the product (the aboria_gb300 package, the
// CUDA library or the C++ headers) links or calls it.  The reference itself
// cannot be compiled here (it requires Boost and Eigen headers), so this file
// restates its arithmetic operation for operation; every function names the
// reference file:line it follows.  It is pinned against the reference's own
// known-answer tests in tests/test_oracle_kats.py (golden values transcribed in
// tests/golden/reference_kats.json).
//
// Build: oracle/build_oracle.sh (g++ -O2 -fopenmp -ffp-contract=off).  FP
// contraction must stay off: the reference's FP64 radius test is evaluated
// without FMA on x86-64, and aarch64 g++ would otherwise fuse a*b+c.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Grid {
  int D;
  double lo[3], hi[3];
  int periodic[3];
  uint32_t size[3];
  double side[3], inv_side[3];
  uint32_t ncells;
};

// CellListOrdered::set_domain_impl, src/CellListOrdered.h:132-186.
void make_grid(Grid &g, int D, const double *lo, const double *hi,
               const int *periodic, double n_leaf, int64_t n_alive) {
  g.D = D;
  for (int d = 0; d < D; ++d) {
    g.lo[d] = lo[d];
    g.hi[d] = hi[d];
    g.periodic[d] = periodic[d];
  }
  const size_t n = (size_t)n_alive;
  if (n_leaf > (double)n) {
    for (int d = 0; d < D; ++d) g.size[d] = 1;
  } else {
    double total_volume = 1.0;
    for (int d = 0; d < D; ++d) total_volume *= (hi[d] - lo[d]);
    const double box_volume = n_leaf / double(n) * total_volume;
    const double box_side = std::pow(box_volume, 1.0 / D);
    for (int d = 0; d < D; ++d) {
      g.size[d] = (unsigned int)std::floor((hi[d] - lo[d]) / box_side);
      if (g.size[d] == 0) g.size[d] = 1;
    }
  }
  g.ncells = 1;
  for (int d = 0; d < D; ++d) {
    g.side[d] = (hi[d] - lo[d]) / g.size[d];
    g.inv_side[d] = 1.0 / g.side[d];  // point_to_bucket_index ctor, SpatialUtil.h:113-116
    g.ncells *= g.size[d];
  }
}

// bucket_index::collapse_index_vector, src/detail/SpatialUtil.h:49-59
// (int vector overload: unsigned multiplier, wraps modulo 2^32).
uint32_t collapse(const Grid &g, const int *v) {
  uint32_t index = 0, mult = 1;
  for (int i = g.D - 1; i >= 0; --i) {
    if (i != g.D - 1) mult *= g.size[i + 1];
    index += mult * (uint32_t)v[i];
  }
  return index;
}

// point_to_bucket_index::find_bucket_index_vector, SpatialUtil.h:125-132.
void bucket_vec(const Grid &g, const double *x, int *v) {
  for (int d = 0; d < g.D; ++d)
    v[d] = (int)std::floor((x[d] - g.lo[d]) * g.inv_side[d]);
}

// distance_helper<2>::norm2, src/detail/Distance.h:132-137 (pow(x,2) == x*x).
inline double norm2(const double *dx, int D) {
  double accum = 0;
  for (int i = 0; i < D; ++i) accum = accum + dx[i] * dx[i];
  return accum;
}

// distance_helper<N> (src/detail/Distance.h:46-137) for the norms of
// euclidean_search (N = 2), manhatten_search (N = 1) and chebyshev_search
// (N = -1, src/Search.h:797-845): the accumulated value (sum of dx^2, sum of
// |dx|, max of |dx|) and its threshold get_value_to_accumulate(r)
// (src/Search.h:184-186): r^2 for N = 2, |r| otherwise.
inline double norm_acc(const double *dx, int D, int lnorm) {
  if (lnorm == 2) return norm2(dx, D);
  double accum = 0;
  for (int i = 0; i < D; ++i) {
    const double a = std::abs(dx[i]);
    accum = lnorm == -1 ? (a > accum ? a : accum) : accum + a;
  }
  return accum;
}
inline double norm_threshold(double r, int lnorm) { return lnorm == 2 ? r * r : std::abs(r); }

// Built-in kernel functors (the closures the reference's tests and the
// benchmark workloads pass to create_sparse_operator / create_dense_operator).
enum {
  K_CONST = 0,
  K_GAUSSIAN = 1,         // exp(-|dx|^2 * p0)
  K_WENDLAND_C2 = 2,      // q=|dx|*p0 ; (1-q)^4 (4q+1), 0 for q>=1
  K_COMPACT_GAUSSIAN = 3, // exp(-p0 * |dx|^2)   (p0 = eps^2)
  K_LAPLACE = 4,          // 1/(|dx| + p0)
  K_MULTIQUADRIC = 5,     // sqrt(|dx|^2 + p0)
  K_SCALAR_SUM = 6,       // row_s[i] + col_s[j]
};

struct KDesc {
  int kind;
  double p[4];
  const double *row_s;
  const double *col_s;
};

inline double kernel_eval(const KDesc &k, const double *dx, int D, int64_t i,
                          int64_t j) {
  double d2 = 0;
  for (int d = 0; d < D; ++d) d2 = d2 + dx[d] * dx[d];
  switch (k.kind) {
  case K_CONST:
    return k.p[0];
  case K_GAUSSIAN:
  case K_COMPACT_GAUSSIAN:
    return std::exp(-d2 * k.p[0]);
  case K_WENDLAND_C2: {
    const double q = std::sqrt(d2) * k.p[0];
    if (q >= 1.0) return 0.0;
    const double t = 1.0 - q;
    const double t2 = t * t;
    return t2 * t2 * (4.0 * q + 1.0);
  }
  case K_LAPLACE:
    return 1.0 / (std::sqrt(d2) + k.p[0]);
  case K_MULTIQUADRIC:
    return std::sqrt(d2 + k.p[0]);
  case K_SCALAR_SUM:
    return k.row_s[i] + k.col_s[j];
  }
  return 0.0;
}

struct CellList {
  Grid g;
  int64_t n;
  const double *pos;  // sorted, n*D
  const uint32_t *begin, *end;
};

// The reference's per-query walk: search_iterator (src/Search.h:150-487) over
// periodic images (lattice order, last dim fastest: src/LatticeIterator.h:269-281)
// x bucket quadrants (lattice_iterator_within_distance,
// src/NeighbourSearchBase.h:1720-2009) x bucket storage order
// (CellListOrderedQuery::get_bucket_particles, src/CellListOrdered.h:472-491),
// with check_candidate's FP64 test (src/Search.h:438-465), in the norm lnorm
// (2, 1 or -1; the domain, bucket and pair tests all use it).
template <class Visit>
void search_walk(const CellList &cl, const double *x, double r, Visit &&visit, int lnorm = 2) {
  const Grid &g = cl.g;
  const int D = g.D;
  const double r2 = norm_threshold(r, lnorm);  // get_value_to_accumulate(r)
  double L[3], half_side[3];
  for (int d = 0; d < D; ++d) {
    L[d] = g.hi[d] - g.lo[d];
    half_side[d] = 0.5 * g.side[d];
  }
  int img_lo[3], img_hi[3], img[3];
  for (int d = 0; d < D; ++d) {
    img_lo[d] = g.periodic[d] ? -1 : 0;
    img_hi[d] = g.periodic[d] ? 2 : 1;
    img[d] = img_lo[d];
  }
  for (;;) {
    double p[3];
    for (int d = 0; d < D; ++d) p[d] = x[d] + img[d] * L[d];
    // outside_domain, NeighbourSearchBase.h:1949-1958
    bool outside;
    {
      double dx[3];
      for (int d = 0; d < D; ++d) {
        const double c = 0.5 * (g.lo[d] + g.hi[d]) - p[d];
        const double hd = 0.5 * (g.hi[d] - g.lo[d]);
        dx[d] = std::max(std::abs(c) - hd, 0.0);
      }
      outside = norm_acc(dx, D, lnorm) > r2;
    }
    if (!outside) {
      auto min_dist = [&](const int *b) {
        double dx[3];
        for (int d = 0; d < D; ++d) {
          const double centre = (b[d] + 0.5) * g.side[d] + g.lo[d];
          dx[d] = std::max(std::abs(centre - p[d]) - half_side[d], 0.0);
        }
        return norm_acc(dx, D, lnorm);
      };
      for (int quadrant = 0; quadrant < (1 << D); ++quadrant) {
        int mn[3], idx[3];
        bool none = false;
        for (int d = 0; d < D; ++d) {
          const bool up = (quadrant >> d) & 1;
          mn[d] = (int)std::floor((p[d] + (up ? 0.5 : -0.5) * g.side[d] - g.lo[d]) *
                                  g.inv_side[d]);
        }
        none = min_dist(mn) > r2;
        if (!none) {
          for (int d = 0; d < D; ++d) {
            const bool up = (quadrant >> d) & 1;
            const int endb = (int)g.size[d] - 1;
            if (up) {
              if (mn[d] < 0) mn[d] = 0;
              else if (mn[d] > endb) { none = true; mn[d] = endb; }
            } else {
              if (mn[d] < 0) { none = true; mn[d] = 0; }
              else if (mn[d] > endb) mn[d] = endb;
            }
          }
        }
        if (none) continue;
        for (int d = 0; d < D; ++d) idx[d] = mn[d];
        for (;;) {
          // visit bucket idx
          const uint32_t b = collapse(g, idx);
          for (uint32_t k = cl.begin[b]; k < cl.end[b]; ++k) {
            const double *pj = cl.pos + (int64_t)k * D;
            double dx[3];
            for (int d = 0; d < D; ++d) dx[d] = pj[d] - p[d];
            if (!(norm_acc(dx, D, lnorm) > r2)) visit((int64_t)k, dx);
          }
          // increment, NeighbourSearchBase.h:1960-2008
          bool valid = false;
          for (int i = D - 1; i >= 0; --i) {
            const bool up = (quadrant >> i) & 1;
            bool pot;
            if (up) { ++idx[i]; pot = idx[i] <= (int)g.size[i] - 1; }
            else { --idx[i]; pot = idx[i] >= 0; }
            if (pot) pot = min_dist(idx) <= r2;
            if (pot) { valid = true; break; }
            idx[i] = mn[i];
          }
          if (!valid) break;
        }
      }
    }
    // next periodic image
    int d = D - 1;
    for (; d >= 0; --d) {
      if (++img[d] < img_hi[d]) break;
      img[d] = img_lo[d];
    }
    if (d < 0) break;
  }
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// Grid dimensions for n_alive particles (set_domain_impl).
uint32_t orc_grid(int D, const double *lo, const double *hi, const int *periodic,
                  double n_leaf, int64_t n_alive, uint32_t *size_out,
                  double *side_out) {
  Grid g;
  make_grid(g, D, lo, hi, periodic, n_leaf, n_alive);
  for (int d = 0; d < D; ++d) {
    size_out[d] = g.size[d];
    side_out[d] = g.side[d];
  }
  return g.ncells;
}

// Unit KATs: collapse_index_vector / reassemble_index_vector
// (src/detail/SpatialUtil.h:49-96).
uint32_t orc_collapse(int D, const uint32_t *size, const int *v) {
  Grid g;
  g.D = D;
  for (int d = 0; d < D; ++d) g.size[d] = size[d];
  // 4-D is needed by the reference KAT; use a local copy of the loop.
  uint32_t index = 0, mult = 1;
  for (int i = D - 1; i >= 0; --i) {
    if (i != D - 1) mult *= size[i + 1];
    index += mult * (uint32_t)v[i];
  }
  return index;
}

void orc_reassemble(int D, const uint32_t *size, uint32_t index, int *v) {
  unsigned int i = index;
  for (int d = D - 1; d >= 0; --d) {
    const double div = (double)i / size[d];
    v[d] = (int)std::round((div - std::floor(div)) * size[d]);
    i = (unsigned int)std::floor(div);
  }
}

// point_to_bucket_index::operator(), SpatialUtil.h:119-138.
int orc_point_to_bucket(int D, const uint32_t *size, const double *lo,
                        const double *side, const double *x, int *v) {
  Grid g;
  g.D = D;
  for (int d = 0; d < D; ++d) {
    g.size[d] = size[d];
    g.lo[d] = lo[d];
    g.side[d] = side[d];
    g.inv_side[d] = 1.0 / side[d];
  }
  bucket_vec(g, x, v);
  return (int)collapse(g, v);
}

// Full cell-list build for a fresh particle set: Particles::init_neighbour_search
// (src/Particles.h:445-456) -> neighbour_search_base::update_positions
// (src/NeighbourSearchBase.h:350-495: enforce_domain_lambda :185-238, alive
// scan/scatter :391-434) -> CellListOrdered::update_positions_impl
// (src/CellListOrdered.h:190-259: hash, sort_by_key, lower/upper_bound) ->
// Particles::reorder (src/Particles.h:694-726).
//
// pos_in: n*D FP64 (AoS).  On return pos_io holds the domain-enforced input
// positions (periodic wrap applied).  Outputs are sized by the caller: pos_out
// and perm_out and keys_out for n entries, begin/end for ncells (orc_grid
// with the alive count; callers pass ncells_cap as capacity).  Returns the
// number of alive particles, or -1 if ncells_cap is too small.
// stable=1: (key, original index) order, the Thrust backend's stable
// sort_by_key (src/detail/Algorithms.h:193-196); stable=0: std::sort with a
// key-only comparison, as the reference's STL backend
// (src/detail/Algorithms.h:173-190).
int64_t orc_celllist_build(int D, int64_t n, double *pos_io, const double *lo,
                           const double *hi, const int *periodic, double n_leaf,
                           int stable, double *pos_out, int64_t *perm_out,
                           uint32_t *keys_out, uint32_t *bucket_begin,
                           uint32_t *bucket_end, uint32_t ncells_cap,
                           uint32_t *size_out, double *side_out, int64_t prev_grid_n,
                           int64_t *grid_n_out) {
  std::vector<uint8_t> alive(n, 1);
  for (int64_t i = 0; i < n; ++i) {
    double *r = pos_io + i * D;
    for (int d = 0; d < D; ++d) {
      if (!std::isfinite(r[d])) {
        alive[i] = 0;
      } else if (periodic[d]) {
        while (r[d] < lo[d]) r[d] += (hi[d] - lo[d]);
        while (r[d] >= hi[d]) r[d] -= (hi[d] - lo[d]);
      } else if ((r[d] < lo[d]) || (r[d] >= hi[d])) {
        alive[i] = 0;
      }
    }
  }
  std::vector<int64_t> alive_idx;
  alive_idx.reserve(n);
  for (int64_t i = 0; i < n; ++i)
    if (alive[i]) alive_idx.push_back(i);
  const int64_t na = (int64_t)alive_idx.size();
  // set_domain_impl recomputes the grid only when the alive count left
  // [0.5, 2] x the count it was last computed with (src/CellListOrdered.h:
  // 133-136); prev_grid_n <= 0 means no grid yet.
  int64_t grid_n = na;
  if (prev_grid_n > 0 && !(na < 0.5 * prev_grid_n || na > 2 * prev_grid_n)) grid_n = prev_grid_n;
  *grid_n_out = grid_n;
  Grid g;
  make_grid(g, D, lo, hi, periodic, n_leaf, grid_n);
  if (g.ncells > ncells_cap) return -1;
  for (int d = 0; d < D; ++d) {
    size_out[d] = g.size[d];
    side_out[d] = g.side[d];
  }
  std::vector<std::pair<uint32_t, int64_t>> kv(na);
  for (int64_t k = 0; k < na; ++k) {
    int v[3];
    bucket_vec(g, pos_io + alive_idx[k] * D, v);
    kv[k] = {collapse(g, v), alive_idx[k]};
  }
  auto cmp = [](const std::pair<uint32_t, int64_t> &a,
                const std::pair<uint32_t, int64_t> &b) { return a.first < b.first; };
  if (stable)
    std::stable_sort(kv.begin(), kv.end(), cmp);
  else
    std::sort(kv.begin(), kv.end(), cmp);
  for (int64_t k = 0; k < na; ++k) {
    keys_out[k] = kv[k].first;
    perm_out[k] = kv[k].second;
    for (int d = 0; d < D; ++d) pos_out[k * D + d] = pos_io[kv[k].second * D + d];
  }
  for (uint32_t c = 0; c < g.ncells; ++c) {
    bucket_begin[c] = (uint32_t)(std::lower_bound(keys_out, keys_out + na, c) - keys_out);
    bucket_end[c] = (uint32_t)(std::upper_bound(keys_out, keys_out + na, c) - keys_out);
  }
  return na;
}

// Neighbour counts of nq query points against a built cell list
// (euclidean_search / manhatten_search / chebyshev_search by lnorm = 2 / 1 /
// -1, src/Search.h:797-845), OpenMP over queries.
void orc_radius_count(int D, const uint32_t *size, const double *lo,
                      const double *hi, const int *periodic, const double *side,
                      int64_t n, const double *pos_sorted, const uint32_t *bbegin,
                      const uint32_t *bend, int64_t nq, const double *q, double r,
                      int lnorm, int32_t *counts) {
  CellList cl;
  Grid &g = cl.g;
  g.D = D;
  g.ncells = 1;
  for (int d = 0; d < D; ++d) {
    g.size[d] = size[d];
    g.lo[d] = lo[d];
    g.hi[d] = hi[d];
    g.periodic[d] = periodic[d];
    g.side[d] = side[d];
    g.inv_side[d] = 1.0 / side[d];
    g.ncells *= size[d];
  }
  cl.n = n;
  cl.pos = pos_sorted;
  cl.begin = bbegin;
  cl.end = bend;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < nq; ++i) {
    int32_t c = 0;
    search_walk(cl, q + i * D, r, [&](int64_t, const double *) { ++c; }, lnorm);
    counts[i] = c;
  }
}

// Neighbour lists in the reference's visiting order, CSR (rowptr from counts),
// in the norm lnorm as for orc_radius_count.
void orc_radius_lists(int D, const uint32_t *size, const double *lo,
                      const double *hi, const int *periodic, const double *side,
                      int64_t n, const double *pos_sorted, const uint32_t *bbegin,
                      const uint32_t *bend, int64_t nq, const double *q, double r,
                      int lnorm, const int64_t *rowptr, int64_t *cols, double *dx_out) {
  CellList cl;
  Grid &g = cl.g;
  g.D = D;
  for (int d = 0; d < D; ++d) {
    g.size[d] = size[d];
    g.lo[d] = lo[d];
    g.hi[d] = hi[d];
    g.periodic[d] = periodic[d];
    g.side[d] = side[d];
    g.inv_side[d] = 1.0 / side[d];
  }
  cl.n = n;
  cl.pos = pos_sorted;
  cl.begin = bbegin;
  cl.end = bend;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < nq; ++i) {
    int64_t o = rowptr[i];
    search_walk(cl, q + i * D, r, [&](int64_t k, const double *dx) {
      cols[o] = k;
      if (dx_out)
        for (int d = 0; d < D; ++d) dx_out[o * D + d] = dx[d];
      ++o;
    }, lnorm);
  }
}

// KernelSparse::evaluate (src/Kernels.h:720-751): c = 0; for each row i (omp
// parallel for, :734-736), for each neighbour j in search order,
// c[i] += f(dx, a_i, b_j) * b[j].  The row particles are the query points.
void orc_sparse_matvec(int D, const uint32_t *size, const double *lo,
                       const double *hi, const int *periodic, const double *side,
                       int64_t ncol, const double *col_pos, const uint32_t *bbegin,
                       const uint32_t *bend, int64_t nrow, const double *row_pos,
                       double r, int kind, const double *params,
                       const double *row_s, const double *col_s, const double *b,
                       double *c) {
  CellList cl;
  Grid &g = cl.g;
  g.D = D;
  for (int d = 0; d < D; ++d) {
    g.size[d] = size[d];
    g.lo[d] = lo[d];
    g.hi[d] = hi[d];
    g.periodic[d] = periodic[d];
    g.side[d] = side[d];
    g.inv_side[d] = 1.0 / side[d];
  }
  cl.n = ncol;
  cl.pos = col_pos;
  cl.begin = bbegin;
  cl.end = bend;
  KDesc k{kind, {params[0], params[1], params[2], params[3]}, row_s, col_s};
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < nrow; ++i) {
    double acc = 0.0;
    search_walk(cl, row_pos + i * D, r, [&](int64_t j, const double *dx) {
      acc += kernel_eval(k, dx, D, i, j) * b[j];
    });
    c[i] = acc;
  }
}

// KernelDense::evaluate (src/Kernels.h:212-239): c[i] = sum_j f(a_i, b_j) b[j]
// in column order; the built-in functors see dx = x_j - x_i.
void orc_dense_matvec(int D, int64_t nrow, const double *row_pos, int64_t ncol,
                      const double *col_pos, int kind, const double *params,
                      const double *row_s, const double *col_s, const double *b,
                      double *c) {
  KDesc k{kind, {params[0], params[1], params[2], params[3]}, row_s, col_s};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nrow; ++i) {
    double acc = 0.0;
    for (int64_t j = 0; j < ncol; ++j) {
      double dx[3];
      for (int d = 0; d < D; ++d) dx[d] = col_pos[j * D + d] - row_pos[i * D + d];
      acc += kernel_eval(k, dx, D, i, j) * b[j];
    }
    c[i] = acc;
  }
}

// Brute-force neighbour counts with periodic images, as the reference's
// tests/neighbours.h:715-765 (brute_force_check, inclusive <= r^2).
void orc_brute_counts(int D, int64_t n, const double *pos, const double *lo,
                      const double *hi, int periodic, double r, int32_t *counts) {
  const double r2 = r * r;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) {
    int32_t c = 0;
    for (int64_t j = 0; j < n; ++j) {
      if (periodic) {
        int img[3] = {-1, -1, -1};
        for (;;) {
          double dx[3];
          for (int d = 0; d < D; ++d)
            dx[d] = pos[j * D + d] - pos[i * D + d] - img[d] * (hi[d] - lo[d]);
          double s = 0;
          for (int d = 0; d < D; ++d) s += dx[d] * dx[d];
          if (s <= r2) ++c;
          int d = D - 1;
          for (; d >= 0; --d) {
            if (++img[d] < 2) break;
            img[d] = -1;
          }
          if (d < 0) break;
        }
      } else {
        double s = 0;
        for (int d = 0; d < D; ++d) {
          const double dx = pos[j * D + d] - pos[i * D + d];
          s += dx * dx;
        }
        if (s <= r2) ++c;
      }
    }
    counts[i] = c;
  }
}

}  // extern "C"

// ------------------------------------------------------------------ octree --
// HyperOctree (src/OctTree.h:168-560): point_to_tag (src/detail/SpatialUtil.h:
// 255-286), stable sort by tag, then build_tree level by level
// (src/OctTree.h:328-475): children of every active node get the tag range
// [mask, mask + 2^((max_level-level)*D) - 1], lower/upper bounds give their
// particle ranges, and a child is EMPTY (no particles), a LEAF (count <= n_leaf
// or last level) or a NODE.
namespace {
int point_to_tag(const double *p, const double *lo, const double *hi, int D, int max_level) {
  double bmin[3], bmax[3];
  for (int i = 0; i < D; ++i) {
    bmin[i] = lo[i];
    bmax[i] = hi[i];
  }
  int result = 0;
  for (int level = 1; level <= max_level; ++level) {
    double mid[3];
    int hi_half[3];
    for (int i = 0; i < D; ++i) {
      mid[i] = 0.5 * (bmin[i] + bmax[i]);
      hi_half[i] = (p[i] < mid[i]) ? 0 : 1;
      result |= hi_half[i];
      result <<= 1;
    }
    for (int i = 0; i < D; ++i) {
      bmin[i] = hi_half[i] ? mid[i] : bmin[i];
      bmax[i] = hi_half[i] ? bmax[i] : mid[i];
    }
  }
  result >>= 1;
  return result;
}
}  // namespace

extern "C" {

// pos: n*D (already domain-enforced; no deletion here).  Outputs: perm (n),
// tags (n, sorted), and the leaves in the reference's order (level by level,
// child order): leaf_level, leaf_tag, leaf_begin, leaf_end (capacity cap).
// Returns the number of leaves (or -1 if cap is too small).
int64_t orc_octree_build(int D, int64_t n, const double *pos, const double *lo, const double *hi,
                         double n_leaf, int64_t *perm, int32_t *tags_out, int32_t *leaf_level,
                         int32_t *leaf_tag, int32_t *leaf_begin, int32_t *leaf_end, int64_t cap) {
  const int max_level = 32 / D - 2;
  const int nchild = 1 << D;
  std::vector<std::pair<int, int64_t>> kv(n);
  for (int64_t i = 0; i < n; ++i) kv[i] = {point_to_tag(pos + i * D, lo, hi, D, max_level), i};
  std::stable_sort(kv.begin(), kv.end(),
                   [](const std::pair<int, int64_t> &a, const std::pair<int, int64_t> &b) {
                     return a.first < b.first;
                   });
  std::vector<int> tags(n);
  for (int64_t i = 0; i < n; ++i) {
    tags[i] = kv[i].first;
    perm[i] = kv[i].second;
    tags_out[i] = kv[i].first;
  }
  std::vector<int> active(1, 0);
  int64_t nleaves = 0;
  for (int level = 1; !active.empty(); ++level) {
    const int shift = (max_level - level) * D;
    const int length = (1 << shift) - 1;
    std::vector<int> next;
    for (int a : active) {
      for (int c = 0; c < nchild; ++c) {
        const int mask = a | (c << shift);
        const int lb = (int)(std::lower_bound(tags.begin(), tags.end(), mask) - tags.begin());
        const int ub = (int)(std::upper_bound(tags.begin(), tags.end(), mask + length) - tags.begin());
        const int count = ub - lb;
        if (count == 0) continue;
        if (level == max_level || count <= n_leaf) {
          if (nleaves >= cap) return -1;
          leaf_level[nleaves] = level;
          leaf_tag[nleaves] = mask;
          leaf_begin[nleaves] = lb;
          leaf_end[nleaves] = ub;
          ++nleaves;
        } else {
          next.push_back(mask);
        }
      }
    }
    active.swap(next);
  }
  return nleaves;
}

}  // extern "C"

// ----------------------------------------------------------------- Schwarz --
// SchwartzPreconditioner (src/Preconditioners.h:1121-1537) restated for the
// oracle: domains from octree leaves (analyze_impl_block :1170-1316), blocks
// assembled with coeff (strict <, periodic-corrected dx: src/detail/Kernels.h:
// 336-368, src/Particles.h:480-496), LU with partial pivoting (the role of
// Eigen's dense solver), and restricted additive application (_solve_impl
// :1477-1522).
namespace {
void leaf_box(int D, const double *lo, const double *hi, int max_level, int level, int tag,
              double *blo, double *bhi) {
  for (int d = 0; d < D; ++d) {
    blo[d] = lo[d];
    bhi[d] = hi[d];
  }
  for (int l = 1; l <= level; ++l)
    for (int d = 0; d < D; ++d) {
      const int bit = (tag >> ((max_level - l) * D + (D - 1 - d))) & 1;
      const double mid = 0.5 * (blo[d] + bhi[d]);
      if (bit) blo[d] = mid; else bhi[d] = mid;
    }
}

void lu_factor(std::vector<double> &A, int n, std::vector<int> &piv) {  // column-major
  piv.resize(n);
  for (int c = 0; c < n; ++c) {
    int p = c;
    double best = std::fabs(A[(size_t)c * n + c]);
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A[(size_t)c * n + r]) > best) {
        best = std::fabs(A[(size_t)c * n + r]);
        p = r;
      }
    piv[c] = p;
    if (p != c)
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)j * n + c], A[(size_t)j * n + p]);
    const double d = A[(size_t)c * n + c];
    if (d != 0.0)
      for (int r = c + 1; r < n; ++r) A[(size_t)c * n + r] /= d;
    for (int j = c + 1; j < n; ++j) {
      const double u = A[(size_t)j * n + c];
      for (int r = c + 1; r < n; ++r) A[(size_t)j * n + r] -= A[(size_t)c * n + r] * u;
    }
  }
}

void lu_solve(const std::vector<double> &A, int n, const std::vector<int> &piv, double *y) {
  for (int c = 0; c < n; ++c)
    if (piv[c] != c) std::swap(y[c], y[piv[c]]);
  for (int c = 0; c < n; ++c)
    for (int r = c + 1; r < n; ++r) y[r] -= A[(size_t)c * n + r] * y[c];
  for (int c = n - 1; c >= 0; --c) {
    y[c] /= A[(size_t)c * n + c];
    for (int r = 0; r < c; ++r) y[r] -= A[(size_t)c * n + r] * y[c];
  }
}
}  // namespace

extern "C" {

// pos: tree-ordered positions (n*D); leaves as returned by orc_octree_build.
void orc_schwarz_apply(int D, int64_t n, const double *pos, const double *lo, const double *hi,
                       const int *periodic, int64_t nleaves, const int32_t *leaf_level,
                       const int32_t *leaf_tag, const int32_t *leaf_begin,
                       const int32_t *leaf_end, double radius, int kind, const double *params,
                       const double *b, double *x) {
  const int max_level = 32 / D - 2;
  const double buf = 1e5 * std::numeric_limits<double>::epsilon();
  KDesc k{kind, {params[0], params[1], params[2], params[3]}, nullptr, nullptr};
  std::vector<double> blo(nleaves * 3), bhi(nleaves * 3);
  for (int64_t l = 0; l < nleaves; ++l)
    leaf_box(D, lo, hi, max_level, leaf_level[l], leaf_tag[l], &blo[l * 3], &bhi[l * 3]);
  for (int64_t i = 0; i < n; ++i) x[i] = b[i];
  const double r2 = radius * radius;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t l = 0; l < nleaves; ++l) {
    if (leaf_end[l] <= leaf_begin[l]) continue;
    std::vector<int64_t> idx;
    for (int64_t i = leaf_begin[l]; i < leaf_end[l]; ++i) idx.push_back(i);
    const size_t own = idx.size();
    for (int64_t m = 0; m < nleaves; ++m) {
      if (m == l) continue;
      bool touch = true;
      for (int d = 0; d < D; ++d)
        if (bhi[m * 3 + d] < blo[l * 3 + d] - buf || blo[m * 3 + d] > bhi[l * 3 + d] + buf)
          touch = false;
      if (touch)
        for (int64_t i = leaf_begin[m]; i < leaf_end[m]; ++i) idx.push_back(i);
    }
    const int nd = (int)idx.size();
    std::vector<double> A((size_t)nd * nd);
    for (int c = 0; c < nd; ++c)
      for (int r = 0; r < nd; ++r) {
        double dx[3], s = 0.0;
        for (int d = 0; d < D; ++d) {
          dx[d] = pos[idx[c] * D + d] - pos[idx[r] * D + d];
          if (periodic[d]) {
            const double w = hi[d] - lo[d];
            while (dx[d] > w / 2) dx[d] -= w;
            while (dx[d] <= -w / 2) dx[d] += w;
          }
          s = s + dx[d] * dx[d];
        }
        A[(size_t)c * nd + r] = s < r2 ? kernel_eval(k, dx, D, 0, 0) : 0.0;
      }
    std::vector<int> piv;
    lu_factor(A, nd, piv);
    std::vector<double> y(nd);
    for (int i = 0; i < nd; ++i) y[i] = b[idx[i]];
    lu_solve(A, nd, piv, y.data());
    for (size_t i = 0; i < own; ++i) x[idx[i]] = y[i];
  }
}

}  // extern "C"

// -------------------------------------------------------------------- FMM --
// Black-box Chebyshev FMM restated from the reference:
//  * BlackBoxExpansions P2M/M2M/M2L/L2L/L2P (src/detail/FastMultipoleMethod.h:
//    96-368), kernel evaluated at Chebyshev node pairs on every call (M2L);
//  * chebyshev_node / chebyshev_Sn (Clenshaw) / ChebyshevRnSingle
//    (src/detail/Chebyshev.h:84-153, 245-294); nodes enumerated in lattice
//    order (last dimension fastest, src/LatticeIterator.h:269-281);
//  * the dual-tree traversal of FastMultipoleMethod::matrix_vector_multiply
//    (src/FastMultipoleMethod.h:111-548) with theta_condition
//    (src/detail/FastMultipoleMethod.h:1249-1279): near iff
//    max_diam^2 > dist^2;
//  * calculate_P2P direct sums (:936-1101).
// The tree is the HyperOctree of orc_octree_build (leaves of <= n_leaf).
namespace {
struct FNode {
  int level, tag, begin, end, kind, first_child;
  double lo[3], hi[3];
};

struct Fmm {
  int D, n, ncheb, nchild;
  std::vector<FNode> nodes;
  std::vector<std::vector<double>> W, g;
  std::vector<std::array<int, 3>> midx;  // multi-index of each Chebyshev node
  const double *pos;                      // tag-sorted positions
  KDesc k;
  double K(const double *a, const double *b) const {
    double dx[3];
    for (int d = 0; d < D; ++d) dx[d] = b[d] - a[d];
    return kernel_eval(k, dx, D, 0, 0);
  }
  double node_pos(int j, int d, const double *lo, const double *hi) const {
    const double c = std::cos((2.0 * midx[j][d] + 1.0) * M_PI / (2.0 * n));
    return 0.5 * (c + 1) * (hi[d] - lo[d]) + lo[d];
  }
  // S_m(x) for m = 0..n-1 per dimension, x in box coordinates
  void sn(const double *p, const double *lo, const double *hi, std::vector<double> &S) const {
    S.assign(n * D, 0.0);
    for (int d = 0; d < D; ++d) {
      const double span = hi[d] - lo[d];
      const double x = span > 0.0 ? (2 * p[d] - lo[d] - hi[d]) / span : 0.0;
      const double invn = 1.0 / n;
      for (int m = 0; m < n; ++m) {
        double b1 = 0.0, b2 = 0.0;
        for (int kk = n - 1; kk >= 1; --kk) {
          const double bk = 2 * invn * std::cos(kk * (2.0 * m + 1.0) * (M_PI / 2) * invn) +
                            2.0 * x * b1 - b2;
          b2 = b1;
          b1 = bk;
        }
        S[m * D + d] = invn + x * b1 - b2;
      }
    }
  }
  double R(const std::vector<double> &S, int j) const {
    double r = 1.0;
    for (int d = 0; d < D; ++d) r *= S[midx[j][d] * D + d];
    return r;
  }
  void upward(int nd, const double *b) {
    FNode &N = nodes[nd];
    std::vector<double> &Wn = W[nd];
    Wn.assign(ncheb, 0.0);
    std::vector<double> S;
    if (N.kind == 1) {
      for (int i = N.begin; i < N.end; ++i) {
        sn(pos + (size_t)i * D, N.lo, N.hi, S);
        for (int j = 0; j < ncheb; ++j) Wn[j] += R(S, j) * b[i];
      }
    } else {
      for (int c = 0; c < nchild; ++c) {
        const int ch = N.first_child + c;
        if (nodes[ch].kind == 0) continue;
        upward(ch, b);
        const FNode &C = nodes[ch];
        for (int j = 0; j < ncheb; ++j) {
          double pj[3];
          for (int d = 0; d < D; ++d) pj[d] = node_pos(j, d, C.lo, C.hi);
          sn(pj, N.lo, N.hi, S);
          for (int i = 0; i < ncheb; ++i) Wn[i] += R(S, i) * W[ch][j];
        }
      }
    }
  }
  bool near(const FNode &t, const FNode &s) const {
    double maxd = std::numeric_limits<double>::min();
    for (int d = 0; d < D; ++d) maxd = std::max(maxd, t.hi[d] - t.lo[d]);
    double dist2 = 0.0;
    for (int d = 0; d < D; ++d) {
      double dd = 0.0;
      if (t.hi[d] < s.lo[d]) dd = s.lo[d] - t.hi[d];
      else if (s.hi[d] < t.lo[d]) dd = t.lo[d] - s.hi[d];
      if (s.hi[d] - s.lo[d] > maxd) maxd = s.hi[d] - s.lo[d];
      dist2 += dd * dd;
    }
    return maxd * maxd > dist2;
  }
  void m2l(int t, int s) {
    const FNode &T = nodes[t], &Sx = nodes[s];
    for (int i = 0; i < ncheb; ++i) {
      double pi[3];
      for (int d = 0; d < D; ++d) pi[d] = node_pos(i, d, T.lo, T.hi);
      double acc = 0.0;
      for (int j = 0; j < ncheb; ++j) {
        double pj[3];
        for (int d = 0; d < D; ++d) pj[d] = node_pos(j, d, Sx.lo, Sx.hi);
        acc += K(pi, pj) * W[s][j];
      }
      g[t][i] += acc;
    }
  }
  void p2p(int t, int s, const double *b, double *c) const {
    const FNode &T = nodes[t], &Sx = nodes[s];
    for (int i = T.begin; i < T.end; ++i)
      for (int j = Sx.begin; j < Sx.end; ++j) c[i] += K(pos + (size_t)i * D, pos + (size_t)j * D) * b[j];
  }
  void leaves_of(int nd, std::vector<int> &out) const {
    if (nodes[nd].kind == 1) { out.push_back(nd); return; }
    if (nodes[nd].kind == 0) return;
    for (int c = 0; c < nchild; ++c) leaves_of(nodes[nd].first_child + c, out);
  }
  void downward(int t, const std::vector<int> &conn_parent, int parent, const double *b, double *c) {
    const FNode &T = nodes[t];
    g[t].assign(ncheb, 0.0);
    std::vector<int> conn;
    std::vector<double> S;
    if (parent < 0) {
      for (int cc = 0; cc < nchild; ++cc) {
        const int s = nodes[0].first_child + cc;
        if (nodes[s].kind == 0) continue;
        if (near(T, nodes[s])) conn.push_back(s); else m2l(t, s);
      }
    } else {
      const FNode &P = nodes[parent];
      for (int i = 0; i < ncheb; ++i) {  // L2L from the parent
        double pi[3];
        for (int d = 0; d < D; ++d) pi[d] = node_pos(i, d, T.lo, T.hi);
        sn(pi, P.lo, P.hi, S);
        double acc = 0.0;
        for (int j = 0; j < ncheb; ++j) acc += R(S, j) * g[parent][j];
        g[t][i] += acc;
      }
      for (int s : conn_parent) {
        if (nodes[s].kind == 1) { conn.push_back(s); continue; }
        for (int cc = 0; cc < nchild; ++cc) {
          const int ch = nodes[s].first_child + cc;
          if (nodes[ch].kind == 0) continue;
          if (near(T, nodes[ch])) conn.push_back(ch); else m2l(t, ch);
        }
      }
    }
    if (T.kind == 2) {
      for (int cc = 0; cc < nchild; ++cc) {
        const int ch = T.first_child + cc;
        if (nodes[ch].kind == 0) continue;
        downward(ch, conn, t, b, c);
      }
    } else {
      for (int i = T.begin; i < T.end; ++i) {  // L2P
        sn(pos + (size_t)i * D, T.lo, T.hi, S);
        double acc = 0.0;
        for (int j = 0; j < ncheb; ++j) acc += R(S, j) * g[t][j];
        c[i] += acc;
      }
      for (int s : conn) {
        std::vector<int> lv;
        leaves_of(s, lv);
        for (int l : lv) p2p(t, l, b, c);
      }
    }
  }
};
}  // namespace

extern "C" {

// Black-box FMM matvec c = K b for positions pos (n*D, any order; output in
// the same order), order n_cheb nodes per dimension, octree leaves <= n_leaf.
void orc_fmm(int D, int n_cheb, int64_t npts, const double *pos_in, const double *lo,
             const double *hi, double n_leaf, int kind, const double *params, const double *b_in,
             double *c_out) {
  Fmm F;
  F.D = D;
  F.n = n_cheb;
  F.nchild = 1 << D;
  F.ncheb = 1;
  for (int d = 0; d < D; ++d) F.ncheb *= n_cheb;
  F.midx.resize(F.ncheb);
  for (int j = 0; j < F.ncheb; ++j) {  // last dimension fastest
    int r = j;
    std::array<int, 3> m{0, 0, 0};
    for (int d = D - 1; d >= 0; --d) {
      m[d] = r % n_cheb;
      r /= n_cheb;
    }
    F.midx[j] = m;
  }
  F.k = KDesc{kind, {params[0], params[1], params[2], params[3]}, nullptr, nullptr};
  const int max_level = 32 / D - 2;
  std::vector<std::pair<int, int64_t>> kv(npts);
  for (int64_t i = 0; i < npts; ++i) kv[i] = {point_to_tag(pos_in + i * D, lo, hi, D, max_level), i};
  std::stable_sort(kv.begin(), kv.end(), [](const std::pair<int, int64_t> &a,
                                            const std::pair<int, int64_t> &b) { return a.first < b.first; });
  std::vector<double> pos(npts * D), b(npts), c(npts, 0.0);
  std::vector<int> tags(npts);
  for (int64_t i = 0; i < npts; ++i) {
    tags[i] = kv[i].first;
    for (int d = 0; d < D; ++d) pos[i * D + d] = pos_in[kv[i].second * D + d];
    b[i] = b_in[kv[i].second];
  }
  F.pos = pos.data();
  // nodes level by level (root = 0), as HyperOctree::build_tree
  FNode root{0, 0, 0, (int)npts, 2, -1, {lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}};
  if (D < 3) for (int d = D; d < 3; ++d) { root.lo[d] = 0; root.hi[d] = 1; }
  F.nodes.push_back(root);
  std::vector<int> active(1, 0);
  for (int level = 1; !active.empty(); ++level) {
    const int shift = (max_level - level) * D;
    const int length = (1 << shift) - 1;
    std::vector<int> next;
    for (int a : active) {
      F.nodes[a].first_child = (int)F.nodes.size();
      for (int ch = 0; ch < F.nchild; ++ch) {
        const int mask = F.nodes[a].tag | (ch << shift);
        const int lb = (int)(std::lower_bound(tags.begin(), tags.end(), mask) - tags.begin());
        const int ub = (int)(std::upper_bound(tags.begin(), tags.end(), mask + length) - tags.begin());
        FNode N{level, mask, lb, ub, 0, -1, {0, 0, 0}, {0, 0, 0}};
        if (ub > lb) N.kind = (level == max_level || (ub - lb) <= n_leaf) ? 1 : 2;
        for (int d = 0; d < 3; ++d) {
          N.lo[d] = F.nodes[a].lo[d];
          N.hi[d] = F.nodes[a].hi[d];
        }
        for (int d = 0; d < D; ++d) {
          const int bit = (ch >> (D - 1 - d)) & 1;
          const double mid = 0.5 * (N.lo[d] + N.hi[d]);
          if (bit) N.lo[d] = mid; else N.hi[d] = mid;
        }
        F.nodes.push_back(N);
        if (N.kind == 2) next.push_back((int)F.nodes.size() - 1);
      }
    }
    active.swap(next);
  }
  F.W.resize(F.nodes.size());
  F.g.resize(F.nodes.size());
  // upward pass from the root's children, then the downward pass
  for (int ch = 0; ch < F.nchild; ++ch) {
    const int s = F.nodes[0].first_child + ch;
    if (F.nodes[s].kind != 0) F.upward(s, b.data());
  }
  std::vector<int> none;
  for (int ch = 0; ch < F.nchild; ++ch) {
    const int t = F.nodes[0].first_child + ch;
    if (F.nodes[t].kind != 0) F.downward(t, none, -1, b.data(), c.data());
  }
  for (int64_t i = 0; i < npts; ++i) c_out[kv[i].second] = c[i];
}

// Direct sum c_i = sum_j K(x_i, x_j) b_j for the targets listed in `targets`.
// skip_self != 0 leaves out j == i: with the regularised Laplace kernel
// 1/(|dx| + 1e-12) the self term 1e12 b_i would otherwise sit in the
// accumulator and round away ~1e-4 of every later term.
void orc_direct_sum(int D, int64_t npts, const double *pos, int kind, const double *params,
                    const double *b, int64_t ntargets, const int64_t *targets, int skip_self,
                    double *c) {
  KDesc k{kind, {params[0], params[1], params[2], params[3]}, nullptr, nullptr};
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t t = 0; t < ntargets; ++t) {
    const int64_t i = targets[t];
    double acc = 0.0;
    for (int64_t j = 0; j < npts; ++j) {
      if (skip_self && j == i) continue;
      double dx[3];
      for (int d = 0; d < D; ++d) dx[d] = pos[j * D + d] - pos[i * D + d];
      acc += kernel_eval(k, dx, D, 0, 0) * b[j];
    }
    c[t] = acc;
  }
}

}  // extern "C"
