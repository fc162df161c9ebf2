/*
 * aboria_gb/Aboria.h -- C++ host layer over the abx C ABI with the names,
 * argument meanings and error behaviour of Aboria's hot-path API:
 *
 *   Particles<std::tuple<...>, D, Storage, SearchMethod>   src/Particles.h:108-112
 *     push_back, size, init_neighbour_search, update_positions, get<position>,
 *     get<id>
 *   CellListOrdered / HyperOctree (search-method tags)       src/CellListOrdered.h, src/OctTree.h
 *   euclidean_search(query, x, r)                            src/Search.h:839-845
 *   create_sparse_operator / create_dense_operator /
 *   create_fmm_operator<N>                                   src/Operators.h:312-515
 *   K * b on any contiguous double vector (Eigen::VectorXd, std::vector<double>)
 *   SchwartzPreconditioner and an Eigen-shaped GMRES         src/Preconditioners.h:1121-1537,
 *                                                            tests/rbf_interpolation.h:360-370
 *
 * Kernel functors.  The built-in closures of the reference's tests and
 * benchmarks are kernel descriptors (Aboria::kernels::*), evaluated by the
 * library's pair kernels.  An arbitrary __host__ __device__ functor
 * f(dx, i, j) -> double is accepted by create_sparse_operator when this header
 * is compiled by nvcc: its matvec runs a kernel instantiated in the caller's
 * translation unit over the FP64 neighbour lists of the radius search
 * (include/aboria_gb/functor_operator.cuh).
 *
 * Errors.  The reference's CHECK prints the message and raises SIGTRAP
 * (src/Log.h:43-81); a non-zero abx status does the same here.  Define
 * ABORIA_GB_THROW before including to get std::runtime_error instead.
 *
 * Storage.  Positions and ids live on the GPU; the host copy that
 * get<position>/get<id> read is refreshed after every call that reorders the
 * particles (init_neighbour_search, update_positions), as the reference's
 * storage is reordered in place (src/Particles.h:694-726).
 */
#ifndef ABORIA_GB_ABORIA_H_
#define ABORIA_GB_ABORIA_H_

#include <array>
#include <csignal>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../abx.h"

#ifdef __CUDACC__
#define ABORIA_GB_HD __host__ __device__
#else
#define ABORIA_GB_HD
#endif

namespace Aboria {

namespace detail {

inline void check(int status, const char *what) {
  if (status == ABX_OK) return;
  const std::string msg = std::string(what) + ": " + abx_last_error() + " (status " +
                          std::to_string(status) + ")";
#ifdef ABORIA_GB_THROW
  throw std::runtime_error(msg);
#else
  std::fprintf(stderr, "CHECK failed: %s\n", msg.c_str());
  std::fflush(stderr);
  std::raise(SIGTRAP);
#endif
}

/* One context (device 0, library-owned stream) shared by every object that is
 * not given one explicitly, like the reference's implicit host/Thrust state. */
class Context {
 public:
  explicit Context(int device = 0, void *stream = nullptr) {
    abx_context *c = nullptr;
    check(abx_context_create(device, stream, &c), "abx_context_create");
    h_ = std::shared_ptr<abx_context>(c, [](abx_context *p) { abx_context_destroy(p); });
  }
  abx_context *get() const { return h_.get(); }

 private:
  std::shared_ptr<abx_context> h_;
};

inline std::shared_ptr<Context> default_context() {
  static std::shared_ptr<Context> ctx = std::make_shared<Context>(0);
  return ctx;
}

}  // namespace detail

/* ------------------------------------------------------------- vectors ---- */
/* Vector<T, N> (src/Vector.h): the fixed-size value type of positions, domain
 * bounds and periodicity flags. */
template <typename T, unsigned int N> struct Vector {
  T v[N];
  ABORIA_GB_HD Vector() : v{} {}
  template <typename... A, typename = typename std::enable_if<sizeof...(A) == N>::type>
  ABORIA_GB_HD Vector(A... a) : v{static_cast<T>(a)...} {}
  ABORIA_GB_HD T &operator[](unsigned i) { return v[i]; }
  ABORIA_GB_HD const T &operator[](unsigned i) const { return v[i]; }
  ABORIA_GB_HD T *data() { return v; }
  ABORIA_GB_HD const T *data() const { return v; }
  ABORIA_GB_HD double squaredNorm() const {
    double s = 0;
    for (unsigned i = 0; i < N; ++i) s += double(v[i]) * double(v[i]);
    return s;
  }
};
typedef Vector<double, 1> vdouble1;
typedef Vector<double, 2> vdouble2;
typedef Vector<double, 3> vdouble3;
typedef Vector<bool, 1> vbool1;
typedef Vector<bool, 2> vbool2;
typedef Vector<bool, 3> vbool3;

/* --------------------------------------------------------------- tags ---- */
struct CellListOrdered {};  // src/CellListOrdered.h (the default search method)
struct HyperOctree {};      // src/OctTree.h

struct position {};  // get<position>(particles) / get<position>(particles)[i]
struct id {};        // get<id>(particles)

/* ----------------------------------------------------------- particles ---- */
template <typename Variables, unsigned int D, typename Storage = void,
          typename SearchMethod = CellListOrdered>
class Particles {
  static_assert(D >= 1 && D <= 3, "the GPU path supports 1 to 3 dimensions");

 public:
  typedef Vector<double, D> double_d;
  typedef Vector<bool, D> bool_d;
  static const unsigned int dimension = D;

  explicit Particles(std::shared_ptr<detail::Context> ctx = detail::default_context())
      : ctx_(std::move(ctx)) {
    abx_particles *p = nullptr;
    detail::check(abx_particles_create(ctx_->get(), int(D), &p), "abx_particles_create");
    h_ = std::shared_ptr<abx_particles>(p, [](abx_particles *q) { abx_particles_destroy(q); });
  }
  /* n particles at the origin (Particles(n) in the reference). */
  explicit Particles(size_t n, std::shared_ptr<detail::Context> ctx = detail::default_context())
      : Particles(std::move(ctx)) {
    pos_.assign(n, double_d());
    for (size_t i = 0; i < n; ++i) ids_.push_back(int64_t(i));
    next_id_ = int64_t(n);
    dirty_ = true;
  }

  size_t size() const { return pos_.size(); }

  /* push_back(position): appended with the next id; takes effect on the
   * device at the next init_neighbour_search / update_positions. */
  void push_back(const double_d &x) {
    pos_.push_back(x);
    ids_.push_back(next_id_++);
    dirty_ = true;
  }

  std::vector<double_d> &positions() { dirty_ = true; return pos_; }
  const std::vector<double_d> &positions() const { return pos_; }
  const std::vector<int64_t> &ids() const { return ids_; }

  /* init_neighbour_search(low, high, periodic, n_particles_in_leaf)
   * (src/Particles.h:445-456): uploads the particles, builds the search
   * structure of SearchMethod and reorders the storage. */
  void init_neighbour_search(const double_d &low, const double_d &high, const bool_d &periodic,
                             double n_particles_in_leaf = 10) {
    upload();
    int per[3] = {0, 0, 0};
    for (unsigned d = 0; d < D; ++d) per[d] = periodic[d] ? 1 : 0;
    low_ = low;
    high_ = high;
    periodic_ = periodic;
    if (std::is_same<SearchMethod, HyperOctree>::value)
      detail::check(abx_particles_init_octree(h_.get(), low.data(), high.data(), per,
                                              n_particles_in_leaf),
                    "init_neighbour_search");
    else
      detail::check(abx_particles_init_neighbour_search(h_.get(), low.data(), high.data(), per,
                                                        n_particles_in_leaf),
                    "init_neighbour_search");
    searched_ = true;
    download();
  }

  /* update_positions() (src/Particles.h:526-540) after the host positions
   * were changed in place: re-enforces the domain and re-sorts. */
  void update_positions() {
    if (!searched_) {
      detail::check(ABX_ERR_STATE, "update_positions before init_neighbour_search");
      return;
    }
    if (int64_t(pos_.size()) != abx_particles_size(h_.get())) {
      detail::check(ABX_ERR_INVALID, "update_positions: particle count changed");
      return;
    }
    detail::check(abx_particles_set_positions(h_.get(), &pos_[0][0]), "set_positions");
    detail::check(abx_particles_update_positions(h_.get()), "update_positions");
    download();
  }

  abx_particles *handle() const { return h_.get(); }
  const std::shared_ptr<detail::Context> &context() const { return ctx_; }
  bool searched() const { return searched_; }
  const double_d &get_min() const { return low_; }
  const double_d &get_max() const { return high_; }
  const bool_d &get_periodic() const { return periodic_; }

 private:
  void upload() {
    if (!dirty_) return;
    const int64_t n = int64_t(pos_.size());
    detail::check(abx_particles_set(h_.get(), n, n ? &pos_[0][0] : nullptr,
                                    n ? ids_.data() : nullptr),
                  "abx_particles_set");
    dirty_ = false;
  }
  void download() {
    const int64_t n = abx_particles_size(h_.get());
    pos_.resize(size_t(n));
    ids_.resize(size_t(n));
    if (n) {
      detail::check(abx_particles_get_positions(h_.get(), &pos_[0][0]), "get_positions");
      detail::check(abx_particles_get_ids(h_.get(), ids_.data()), "get_ids");
    }
    dirty_ = false;
  }

  static_assert(sizeof(Vector<double, D>) == D * sizeof(double), "packed positions");
  std::shared_ptr<detail::Context> ctx_;
  std::shared_ptr<abx_particles> h_;
  std::vector<double_d> pos_;
  std::vector<int64_t> ids_;
  double_d low_, high_;
  bool_d periodic_;
  int64_t next_id_ = 0;
  bool dirty_ = true;
  bool searched_ = false;
};

namespace detail {
template <typename Tag> struct getter;
template <> struct getter<position> {
  template <typename P> static decltype(auto) get(P &p) { return p.positions(); }
};
template <> struct getter<id> {
  template <typename P> static const std::vector<int64_t> &get(P &p) { return p.ids(); }
};
}  // namespace detail

/* get<position>(particles)[i] / get<id>(particles)[i] (src/Get.h). */
template <typename Tag, typename P> decltype(auto) get(P &p) {
  return detail::getter<Tag>::get(p);
}

/* ----------------------------------------------------- radius search ---- */
/* One neighbour of euclidean_search: storage index j of the particle and
 * dx = x_j - x (periodic image applied), as the reference's search iterator
 * exposes them (src/Search.h:64-496). */
template <unsigned int D> struct SearchResult {
  int32_t index;
  Vector<double, D> dx;
};

/* euclidean_search(particles.get_query(), x, r) (src/Search.h:839-845): every
 * particle (and periodic image) with |x_j - x|^2 <= r^2 in FP64.  One query
 * per call; many queries belong in abx_radius_count / abx_radius_query_csr. */
template <typename P>
std::vector<SearchResult<P::dimension>> euclidean_search(const P &particles,
                                                         const typename P::double_d &x,
                                                         double r) {
  constexpr unsigned D = P::dimension;
  std::vector<SearchResult<D>> out;
  if (!particles.searched()) {
    detail::check(ABX_ERR_STATE, "euclidean_search before init_neighbour_search");
    return out;
  }
  int64_t rowptr[2] = {0, 0};
  detail::check(abx_radius_query_csr(particles.handle(), 1, x.data(), r, rowptr, nullptr, 0),
                "euclidean_search");
  std::vector<int32_t> cols(static_cast<size_t>(rowptr[1]));
  if (!cols.empty())
    detail::check(abx_radius_query_csr(particles.handle(), 1, x.data(), r, rowptr, cols.data(),
                                       rowptr[1]),
                  "euclidean_search");
  // dx from the storage positions with the minimum periodic image, which is
  // the image the search accepted whenever r is below half the domain width
  const auto &pos = particles.positions();
  for (int32_t j : cols) {
    SearchResult<D> s;
    s.index = j;
    for (unsigned d = 0; d < D; ++d) {
      double dx = pos[size_t(j)][d] - x[d];
      if (particles.get_periodic()[d]) {
        const double w = particles.get_max()[d] - particles.get_min()[d];
        while (dx > w / 2) dx -= w;
        while (dx <= -w / 2) dx += w;
      }
      s.dx[d] = dx;
    }
    out.push_back(s);
  }
  return out;
}

/* ---------------------------------------------------- kernel functors ---- */
/* The closures of the reference's examples as descriptors for the library's
 * pair kernels (abx.h ABX_K_*). */
namespace kernels {
inline abx_kernel make(int kind, double p0 = 0, double p1 = 0) {
  abx_kernel k{};
  k.kind = kind;
  k.p[0] = p0;
  k.p[1] = p1;
  return k;
}
/* exp(-|dx|^2 / c^2) */
inline abx_kernel gaussian(double c) { return make(ABX_K_GAUSSIAN, 1.0 / (c * c)); }
/* q = |dx| / r: (1-q)^4 (4q+1), 0 for q >= 1 */
inline abx_kernel wendland_c2(double r) { return make(ABX_K_WENDLAND_C2, 1.0 / r); }
/* exp(-(eps |dx|)^2), used inside a cut-off radius */
inline abx_kernel compact_gaussian(double eps) { return make(ABX_K_COMPACT_GAUSSIAN, eps * eps); }
/* 1 / (|dx| + delta) */
inline abx_kernel laplace(double delta = 1e-12) { return make(ABX_K_LAPLACE, delta); }
/* sqrt(|dx|^2 + c2) */
inline abx_kernel multiquadric(double c2) { return make(ABX_K_MULTIQUADRIC, c2); }
inline abx_kernel constant(double v) { return make(ABX_K_CONST, v); }
}  // namespace kernels

/* ------------------------------------------------------------ operators ---- */
/* MatrixReplacement (src/Operators.h:75-281): a matrix-free kernel operator.
 * It refers to its particle sets (src/Kernels.h:133-135), which must outlive it. */
class Operator {
 public:
  Operator() = default;
  explicit Operator(abx_operator *h)
      : h_(h, [](abx_operator *p) { abx_operator_destroy(p); }) {}

  int64_t rows() const { return abx_operator_rows(h_.get()); }
  int64_t cols() const { return abx_operator_cols(h_.get()); }

  /* ABX_PREC_FP64 (default) or ABX_PREC_MIXED. */
  Operator &set_precision(int mode) {
    detail::check(abx_operator_set_precision(h_.get(), mode), "set_precision");
    return *this;
  }

  /* c = K * b into caller storage (host or device pointers). */
  void apply(const double *b, double *c) const {
    detail::check(abx_operator_matvec(h_.get(), b, c), "K*b");
  }

  /* K * b for any vector type with data(), size() and a size constructor
   * (Eigen::VectorXd, std::vector<double>). */
  template <typename Vec> Vec operator*(const Vec &b) const {
    if (int64_t(b.size()) != cols()) {
      detail::check(ABX_ERR_INVALID, "K*b: size of b does not match the operator's columns");
      return Vec();
    }
    Vec c(static_cast<size_t>(rows()));
    apply(b.data(), c.data());
    return c;
  }

  abx_operator *handle() const { return h_.get(); }

 protected:
  std::shared_ptr<abx_operator> h_;
};

template <typename RowP, typename ColP>
Operator create_sparse_operator(const RowP &row_particles, const ColP &col_particles,
                                double radius, const abx_kernel &kernel) {
  abx_operator *h = nullptr;
  detail::check(abx_create_sparse_operator(row_particles.handle(), col_particles.handle(), radius,
                                           &kernel, &h),
                "create_sparse_operator");
  return Operator(h);
}

template <typename RowP, typename ColP>
Operator create_dense_operator(const RowP &row_particles, const ColP &col_particles,
                               const abx_kernel &kernel) {
  abx_operator *h = nullptr;
  detail::check(abx_create_dense_operator(row_particles.handle(), col_particles.handle(), &kernel,
                                          &h),
                "create_dense_operator");
  return Operator(h);
}

/* create_fmm_operator<N>(rows, cols, kernel): Chebyshev order N on the
 * HyperOctree of the particle set (rows and cols the same set, as in the
 * reference's tests/fmm.h). */
template <unsigned int N, typename RowP, typename ColP>
Operator create_fmm_operator(const RowP &row_particles, const ColP &col_particles,
                             const abx_kernel &kernel) {
  if (row_particles.handle() != col_particles.handle()) {
    detail::check(ABX_ERR_INVALID, "create_fmm_operator: rows and cols must be one particle set");
    return Operator();
  }
  abx_operator *h = nullptr;
  detail::check(abx_create_fmm_operator(row_particles.handle(), &kernel, int(N), &h),
                "create_fmm_operator");
  return Operator(h);
}

/* -------------------------------------------------------------- solvers ---- */
/* SchwartzPreconditioner<Solver> (src/Preconditioners.h:1121-1537): domains
 * are the octree leaves of the operator's particle set; blocks are factorised
 * by FP64 LU whatever Solver names (LLT, LU, ...). */
template <typename Solver = void> class SchwartzPreconditioner {
 public:
  void analyzePattern(const Operator &op) { op_ = &op; }
  SchwartzPreconditioner &factorize(const Operator &op) {
    abx_precond *h = nullptr;
    detail::check(abx_precond_create_schwarz(op.handle(), ABX_PREC_FP64, &h),
                  "SchwartzPreconditioner::factorize");
    h_ = std::shared_ptr<abx_precond>(h, [](abx_precond *p) { abx_precond_destroy(p); });
    return *this;
  }
  SchwartzPreconditioner &compute(const Operator &op) {
    analyzePattern(op);
    return factorize(op);
  }
  template <typename Vec> Vec solve(const Vec &b) const {
    Vec x(static_cast<size_t>(b.size()));
    detail::check(abx_precond_apply(h_.get(), b.data(), x.data()), "SchwartzPreconditioner::solve");
    return x;
  }
  abx_precond *handle() const { return h_.get(); }

 private:
  const Operator *op_ = nullptr;
  std::shared_ptr<abx_precond> h_;
};

/* Eigen::GMRES<MatrixReplacement, Preconditioner>-shaped restarted GMRES
 * (flexible, right-preconditioned, FP64 Gram-Schmidt and Givens). */
template <typename Op = Operator, typename Preconditioner = SchwartzPreconditioner<>>
class GMRES {
 public:
  void set_restart(int r) { restart_ = r; }
  void setMaxIterations(int n) { max_iters_ = n; }
  void setTolerance(double t) { tol_ = t; }
  Preconditioner &preconditioner() { return pc_; }
  GMRES &compute(const Op &op) {
    op_ = &op;
    pc_.compute(op);
    return *this;
  }
  template <typename Vec> Vec solve(const Vec &b) {
    Vec x(static_cast<size_t>(b.size()));
    for (size_t i = 0; i < size_t(b.size()); ++i) x[i] = 0.0;
    detail::check(abx_gmres_solve(op_->handle(), nullptr, pc_.handle(), b.data(), x.data(),
                                  restart_, max_iters_, tol_, &iters_, &err_),
                  "GMRES::solve");
    return x;
  }
  int iterations() const { return iters_; }
  double error() const { return err_; }

 private:
  const Op *op_ = nullptr;
  Preconditioner pc_;
  int restart_ = 30;
  int max_iters_ = 1000;
  double tol_ = 1e-12;
  int iters_ = 0;
  double err_ = 0;
};

}  // namespace Aboria

#ifdef __CUDACC__
#include "functor_operator.cuh"
#endif

#endif  // ABORIA_GB_ABORIA_H_
