/*
 * aboria_gb/functor_operator.cuh -- operators built from the reference's
 * closures, for translation units compiled by nvcc (included by
 * aboria_gb/Aboria.h under __CUDACC__).
 *
 *   create_sparse_operator(rows, cols, r, f)       KernelSparseConst   src/Kernels.h:754-776
 *   create_sparse_operator(rows, cols, r(a), f)    KernelSparse        src/Kernels.h:692-751
 *   create_dense_operator(rows, cols, f)           KernelDense         src/Kernels.h:138-268
 *
 * The closures are __host__ __device__ functors with the reference's
 * arguments: f(dx, a, b) for the sparse operators, f(a, b) for the dense one,
 * a and b particle references (Particles::const_reference) read with
 * get<position>, get<id> and get<variable>; r(a) gives the search radius of
 * row a.  (The sparse form f(dx, i, j) with storage indices is accepted too.)
 * Each K * b runs a kernel instantiated here for the functor, matrix-free:
 *
 *   sparse: one warp per row walks the buckets of the column set's
 *     CellListOrdered grid (the library's, abx_particles_get_view) that can
 *     hold a neighbour, including periodic images, and applies the
 *     reference's FP64 test !(((0+dx0^2)+dx1^2)+dx2^2 > r^2) with
 *     dx = x_j - (x_i + image*L) (src/Search.h:188-190, 438-465) -- the dx
 *     handed to f is that of the accepted image; sum f * b_j in FP64.
 *   dense: one thread per row, every column, sum f(a, b) * b_j in FP64.
 *
 * A functor returning Vector<double, BR> gives BR rows per particle (the
 * reference's block kernels returning an Eigen BR x 1 block).  The particle
 * columns (positions, ids, variables) are copied to the device when the host
 * storage changed since the last K * b.  Kernels and copies run on the legacy
 * default stream.
 */
#ifndef ABORIA_GB_FUNCTOR_OPERATOR_CUH_
#define ABORIA_GB_FUNCTOR_OPERATOR_CUH_

#include <cuda_runtime.h>

namespace Aboria {
namespace detail {

inline void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
#ifdef ABORIA_GB_THROW
    throw std::runtime_error(m);
#else
    std::fprintf(stderr, "CHECK failed: %s\n", m.c_str());
    std::fflush(stderr);
    std::raise(SIGTRAP);
#endif
  }
}

template <typename T> struct DeviceArray {
  T *ptr = nullptr;
  explicit DeviceArray(size_t n) {
    if (n) check_cuda(cudaMalloc(&ptr, n * sizeof(T)), "cudaMalloc");
  }
  ~DeviceArray() {
    if (ptr) cudaFree(ptr);
  }
  DeviceArray(const DeviceArray &) = delete;
  DeviceArray &operator=(const DeviceArray &) = delete;
};

// Rows of a functor's value: 1 for a double, BR for Vector<double, BR>.
template <typename R> struct BlockRows {
  static constexpr unsigned value = 1;
  static __host__ __device__ double get(const R &r, unsigned) { return r; }
};
template <unsigned BR> struct BlockRows<Vector<double, BR>> {
  static constexpr unsigned value = BR;
  static __host__ __device__ double get(const Vector<double, BR> &r, unsigned k) { return r[k]; }
};

// Device copies of one particle set's columns, refreshed when its host
// storage version moved.
struct DeviceColumns {
  uint64_t version = ~uint64_t(0);
  std::shared_ptr<DeviceArray<double>> pos;   // SoA
  std::shared_ptr<DeviceArray<int64_t>> ids;
  std::vector<std::shared_ptr<DeviceArray<unsigned char>>> vars;
};

template <typename T> void upload(std::shared_ptr<DeviceArray<unsigned char>> &dst,
                                  const std::vector<T> &src) {
  dst = std::make_shared<DeviceArray<unsigned char>>(src.size() * sizeof(T));
  if (!src.empty())
    check_cuda(cudaMemcpy(dst->ptr, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice),
               "cudaMemcpy");
}

// The particle reference of row/column 0 of a particle set (index set per
// pair in the kernels), with the device columns brought up to date.
template <typename P> typename P::const_reference device_ref(const P &p) {
  constexpr unsigned D = P::dimension;
  std::shared_ptr<void> &cache = p.device_cache();
  if (!cache) cache = std::make_shared<DeviceColumns>();
  DeviceColumns &dc = *static_cast<DeviceColumns *>(cache.get());
  const size_t n = p.size();
  if (dc.version != p.version()) {
    std::vector<double> soa(n * D);
    for (size_t i = 0; i < n; ++i)
      for (unsigned d = 0; d < D; ++d) soa[d * n + i] = p.positions()[i][d];
    dc.pos = std::make_shared<DeviceArray<double>>(soa.size());
    dc.ids = std::make_shared<DeviceArray<int64_t>>(n);
    if (n) {
      check_cuda(cudaMemcpy(dc.pos->ptr, soa.data(), soa.size() * 8, cudaMemcpyHostToDevice),
                 "cudaMemcpy");
      check_cuda(cudaMemcpy(dc.ids->ptr, p.ids().data(), n * 8, cudaMemcpyHostToDevice),
                 "cudaMemcpy");
    }
    dc.vars.clear();
    std::apply([&dc](const auto &...col) {
      int dummy[] = {0, (dc.vars.emplace_back(), upload(dc.vars.back(), col), 0)...};
      (void)dummy;
    }, p.variables());
    dc.version = p.version();
  }
  typename P::const_reference r{};
  r.pos = dc.pos->ptr;
  r.n = int64_t(n);
  r.ids = dc.ids->ptr;
  for (size_t k = 0; k < dc.vars.size(); ++k) r.vars[k] = dc.vars[k]->ptr;
  r.index = 0;
  return r;
}

// The column set's CellListOrdered grid for the bucket walk.
struct CellGrid {
  int dim;
  uint32_t size[3];
  double lo[3], side[3], L[3];
  int periodic[3];
  const uint32_t *bb, *be;
};

inline CellGrid cell_grid(abx_particles *h, int64_t n_expected) {
  abx_particles_view v;
  check(abx_particles_get_view(h, &v), "abx_particles_get_view");
  CellGrid g{};
  if (v.search_kind != 0) {
    check(ABX_ERR_STATE, "user-functor sparse operators search a CellListOrdered particle set");
    return g;
  }
  if (v.n != n_expected) {
    check(ABX_ERR_STATE, "the column particles changed since init_neighbour_search");
    return g;
  }
  g.dim = v.dim;
  for (int d = 0; d < 3; ++d) {
    g.size[d] = v.size[d];
    g.lo[d] = v.lo[d];
    g.side[d] = v.side[d];
    g.L[d] = v.hi[d] - v.lo[d];
    g.periodic[d] = v.periodic[d];
  }
  g.bb = v.bucket_begin;
  g.be = v.bucket_end;
  return g;
}

template <typename F, typename R, typename C, unsigned D>
using sparse_ref_result = decltype(std::declval<F>()(Vector<double, D>(), std::declval<R>(),
                                                     std::declval<C>()));
template <typename F, unsigned D>
using sparse_index_result = decltype(std::declval<F>()(Vector<double, D>(), int64_t(0), int64_t(0)));

template <typename F, typename R, typename C, unsigned D, typename = void>
struct takes_refs : std::false_type {};
template <typename F, typename R, typename C, unsigned D>
struct takes_refs<F, R, C, D, std::void_t<sparse_ref_result<F, R, C, D>>> : std::true_type {};

// f(dx, a, b) (the reference's closure) or f(dx, i, j) (storage indices)
template <bool REFS> struct SparseCall;
template <> struct SparseCall<true> {
  template <typename F, typename V, typename R, typename C>
  static __host__ __device__ auto call(const F &f, const V &dx, const R &a, const C &b) {
    return f(dx, a, b);
  }
};
template <> struct SparseCall<false> {
  template <typename F, typename V, typename R, typename C>
  static __host__ __device__ auto call(const F &f, const V &dx, const R &a, const C &b) {
    return f(dx, a.index, b.index);
  }
};

struct CountPair {
  template <typename V> __host__ __device__ double operator()(const V &, int64_t, int64_t) const {
    return 1.0;
  }
};

struct ConstRadius {
  double r;
  template <typename R> __host__ __device__ double operator()(const R &) const { return r; }
};

// NORM: the search norm, 2 euclidean (accumulate dx^2, compare with r^2), 1
// manhattan (accumulate |dx|), -1 chebyshev (max |dx|), compared with r
// (src/detail/Distance.h:46-137)
template <unsigned D, bool REFS, typename RowRef, typename ColRef, typename F, typename RF,
          int NORM = 2>
__global__ void functor_sparse_walk(RowRef rbase, ColRef cbase, CellGrid g, F f, RF rf,
                                    const double *__restrict__ b, double *__restrict__ c,
                                    int64_t nrows) {
  using R = decltype(SparseCall<REFS>::call(f, Vector<double, D>(), rbase, cbase));
  constexpr unsigned BR = BlockRows<R>::value;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= nrows) return;
  RowRef a = rbase;
  a.index = i;
  double xi[D];
  for (unsigned d = 0; d < D; ++d) xi[d] = a.pos[d * a.n + i];
  const double r = rf(a);
  const double r2 = NORM == 2 ? r * r : r;  // get_value_to_accumulate(r)
  // buckets that may hold a neighbour (one extra bucket each side covers the
  // rounding of the bucket assignment), images -1, 0, +1
  int ulo[3] = {0, 0, 0}, uhi[3] = {0, 0, 0};
  int64_t nbox = 1;
  for (unsigned d = 0; d < D; ++d) {
    const int sz = (int)g.size[d];
    double a0 = floor((xi[d] - r - g.lo[d]) / g.side[d]) - 1.0;
    double a1 = floor((xi[d] + r - g.lo[d]) / g.side[d]) + 1.0;
    const double mn = g.periodic[d] ? -sz : 0.0, mx = g.periodic[d] ? 2.0 * sz - 1.0 : sz - 1.0;
    a0 = a0 < mn ? mn : a0;
    a1 = a1 > mx ? mx : a1;
    if (!(a0 <= a1)) nbox = 0;
    ulo[d] = (int)(a0 <= a1 ? a0 : 0.0);
    uhi[d] = (int)(a0 <= a1 ? a1 : -1.0);
    nbox *= (int64_t)(uhi[d] - ulo[d] + 1);
  }
  double acc[BR];
  for (unsigned k = 0; k < BR; ++k) acc[k] = 0.0;
  for (int64_t t = 0; t < nbox; ++t) {
    int64_t rem = t;
    uint32_t key = 0;
    double shift[D];
    for (int d = (int)D - 1; d >= 0; --d) {
      const int len = uhi[d] - ulo[d] + 1;
      const int u = ulo[d] + (int)(rem % len);
      rem /= len;
      const int sz = (int)g.size[d];
      int w = u, img = 0;
      if (u < 0) {
        w = u + sz;
        img = 1;
      } else if (u >= sz) {
        w = u - sz;
        img = -1;
      }
      shift[d] = __dmul_rn((double)img, g.L[d]);
      uint32_t mult = 1;
      for (unsigned e = d + 1; e < D; ++e) mult *= g.size[e];
      key += (uint32_t)w * mult;
    }
    double cur[D];
    for (unsigned d = 0; d < D; ++d) cur[d] = __dadd_rn(xi[d], shift[d]);
    const uint32_t j0 = g.bb[key], j1 = g.be[key];
    for (uint32_t j = j0 + lane; j < j1; j += 32) {
      Vector<double, D> dx;
      double acc2 = 0.0;
      for (unsigned d = 0; d < D; ++d) {
        dx[d] = __dsub_rn(cbase.pos[d * cbase.n + j], cur[d]);
        if (NORM == 2)
          acc2 = __dadd_rn(acc2, __dmul_rn(dx[d], dx[d]));
        else if (NORM == 1)
          acc2 = __dadd_rn(acc2, fabs(dx[d]));
        else
          acc2 = fmax(acc2, fabs(dx[d]));
      }
      if (!(acc2 > r2)) {
        ColRef bj = cbase;
        bj.index = j;
        const R v = SparseCall<REFS>::call(f, dx, a, bj);
        for (unsigned k = 0; k < BR; ++k) acc[k] += BlockRows<R>::get(v, k) * b[j];
      }
    }
  }
  for (unsigned k = 0; k < BR; ++k) {
    double s = acc[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) c[i * BR + k] = s;
  }
}

template <typename RowRef, typename ColRef, typename F>
__global__ void functor_dense(RowRef rbase, ColRef cbase, F f, const double *__restrict__ b,
                              double *__restrict__ c, int64_t nrows, int64_t ncols) {
  using R = decltype(f(rbase, cbase));
  constexpr unsigned BR = BlockRows<R>::value;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  RowRef a = rbase;
  a.index = i;
  double acc[BR];
  for (unsigned k = 0; k < BR; ++k) acc[k] = 0.0;
  for (int64_t j = 0; j < ncols; ++j) {
    ColRef bj = cbase;
    bj.index = j;
    const R v = f(a, bj);
    for (unsigned k = 0; k < BR; ++k) acc[k] += BlockRows<R>::get(v, k) * b[j];
  }
  for (unsigned k = 0; k < BR; ++k) c[i * BR + k] = acc[k];
}

}  // namespace detail

/* The operator of a user closure; K * b like Aboria::Operator.  It refers to
 * its particle sets, which must outlive it (src/Kernels.h:133-135). */
template <typename RowP, typename ColP, typename F, typename RF, bool DENSE, int NORM = 2>
class FunctorOperator {
  static constexpr unsigned D = RowP::dimension;
  typedef typename RowP::const_reference RowRef;
  typedef typename ColP::const_reference ColRef;
  static constexpr bool REFS = detail::takes_refs<F, RowRef, ColRef, D>::value;
  template <bool DN, int = 0> struct Result {
    typedef decltype(detail::SparseCall<REFS>::call(std::declval<F>(), Vector<double, D>(),
                                                    std::declval<RowRef>(),
                                                    std::declval<ColRef>())) type;
  };
  template <int Z> struct Result<true, Z> {
    typedef decltype(std::declval<F>()(std::declval<RowRef>(), std::declval<ColRef>())) type;
  };

 public:
  static constexpr unsigned block_rows = detail::BlockRows<typename Result<DENSE>::type>::value;

  FunctorOperator(const RowP &rows, const ColP &cols, RF rf, F f)
      : rows_(&rows), cols_(&cols), f_(f), rf_(rf) {
    static_assert(RowP::dimension == ColP::dimension, "dimension mismatch");
    if (!DENSE && !cols.searched())
      detail::check(ABX_ERR_STATE, "create_sparse_operator before init_neighbour_search");
  }

  int64_t rows() const { return int64_t(rows_->size()) * block_rows; }
  int64_t cols() const { return int64_t(cols_->size()); }

  /* c = K * b with b and c in device memory, on the legacy default stream. */
  void apply_device(const double *b, double *c) const {
    const int64_t nr = int64_t(rows_->size()), nc = int64_t(cols_->size());
    if (nr == 0) return;
    if (nc == 0) {
      detail::check_cuda(cudaMemset(c, 0, size_t(nr) * block_rows * sizeof(double)), "cudaMemset");
      return;
    }
    const RowRef a = detail::device_ref(*rows_);
    const ColRef bref = detail::device_ref(*cols_);
    const int threads = 256;
    if constexpr (DENSE) {
      detail::functor_dense<<<(unsigned)((nr + threads - 1) / threads), threads>>>(a, bref, f_, b,
                                                                                 c, nr, nc);
    } else {
      const detail::CellGrid g = detail::cell_grid(cols_->handle(), nc);
      detail::functor_sparse_walk<D, REFS, RowRef, ColRef, F, RF, NORM>
          <<<(unsigned)((nr * 32 + threads - 1) / threads), threads>>>(a, bref, g, f_, rf_, b, c,
                                                                      nr);
    }
    detail::check_cuda(cudaGetLastError(), "user-functor operator launch");
  }

  /* c = K * b with host b and c. */
  void apply(const double *b, double *c) const {
    const size_t nr = size_t(rows()), nc = size_t(cols());
    detail::DeviceArray<double> db(nc), dc(nr);
    if (nc)
      detail::check_cuda(cudaMemcpy(db.ptr, b, nc * sizeof(double), cudaMemcpyHostToDevice),
                         "cudaMemcpy");
    apply_device(db.ptr, dc.ptr);
    if (nr)
      detail::check_cuda(cudaMemcpy(c, dc.ptr, nr * sizeof(double), cudaMemcpyDeviceToHost),
                         "cudaMemcpy");
  }

  template <typename Vec> Vec operator*(const Vec &b) const {
    if (int64_t(b.size()) != cols()) {
      detail::check(ABX_ERR_INVALID, "K*b: size of b does not match the operator's columns");
      return Vec();
    }
    Vec c(static_cast<size_t>(rows()));
    apply(b.data(), c.data());
    return c;
  }

  /* pairs within the search radius (every pair for the dense operator) times
   * the block size: the nonzeros of the reference's assembled matrix */
  int64_t nonzeros() const {
    const int64_t nr = int64_t(rows_->size()), nc = int64_t(cols_->size());
    if constexpr (DENSE) {
      return nr * nc * block_rows;
    } else {
    if (nr == 0 || nc == 0) return 0;
    detail::DeviceArray<double> ones(static_cast<size_t>(nc)), cnt(static_cast<size_t>(nr));
    std::vector<double> h(static_cast<size_t>(nc), 1.0);
    detail::check_cuda(cudaMemcpy(ones.ptr, h.data(), size_t(nc) * 8, cudaMemcpyHostToDevice),
                       "cudaMemcpy");
    const RowRef a = detail::device_ref(*rows_);
    const ColRef bref = detail::device_ref(*cols_);
    const detail::CellGrid g = detail::cell_grid(cols_->handle(), nc);
    const int threads = 256;
    detail::functor_sparse_walk<D, false, RowRef, ColRef, detail::CountPair, RF, NORM>
        <<<(unsigned)((nr * 32 + threads - 1) / threads), threads>>>(
            a, bref, g, detail::CountPair{}, rf_, ones.ptr, cnt.ptr, nr);
    detail::check_cuda(cudaGetLastError(), "pair count launch");
    std::vector<double> c(static_cast<size_t>(nr));
    detail::check_cuda(cudaMemcpy(c.data(), cnt.ptr, size_t(nr) * 8, cudaMemcpyDeviceToHost),
                       "cudaMemcpy");
    double total = 0;
    for (double v : c) total += v;
    return int64_t(total) * block_rows;
    }
  }

 private:
  const RowP *rows_;
  const ColP *cols_;
  F f_;
  RF rf_;
};

/* create_sparse_operator(rows, cols, radius, f) with a __host__ __device__
 * closure f(dx, a, b) (src/Operators.h:478-515, KernelSparseConst). */
template <typename RowP, typename ColP, typename F,
          typename = typename std::enable_if<
              !std::is_same<typename std::decay<F>::type, abx_kernel>::value>::type>
FunctorOperator<RowP, ColP, F, detail::ConstRadius, false>
create_sparse_operator(const RowP &row_particles, const ColP &col_particles, double radius, F f) {
  return FunctorOperator<RowP, ColP, F, detail::ConstRadius, false>(
      row_particles, col_particles, detail::ConstRadius{radius}, f);
}

/* create_sparse_operator(rows, cols, radius_function, f): the search radius
 * of row a is radius_function(a) (src/Operators.h:472-484, the
 * m_radius_function(ai) of src/Kernels.h:738). */
template <typename RowP, typename ColP, typename RF, typename F,
          typename = typename std::enable_if<!std::is_convertible<RF, double>::value>::type>
FunctorOperator<RowP, ColP, F, RF, false>
create_sparse_operator(const RowP &row_particles, const ColP &col_particles, RF radius_function,
                       F f) {
  return FunctorOperator<RowP, ColP, F, RF, false>(row_particles, col_particles, radius_function,
                                                   f);
}

/* create_dense_operator(rows, cols, f) with a __host__ __device__ closure
 * f(a, b) (src/Operators.h:312-318, KernelDense). */
template <typename RowP, typename ColP, typename F,
          typename = typename std::enable_if<
              !std::is_same<typename std::decay<F>::type, abx_kernel>::value>::type>
FunctorOperator<RowP, ColP, F, detail::ConstRadius, true>
create_dense_operator(const RowP &row_particles, const ColP &col_particles, F f) {
  return FunctorOperator<RowP, ColP, F, detail::ConstRadius, true>(
      row_particles, col_particles, detail::ConstRadius{0.0}, f);
}

}  // namespace Aboria

#endif  // ABORIA_GB_FUNCTOR_OPERATOR_CUH_
