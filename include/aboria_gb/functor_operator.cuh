/*
 * aboria_gb/functor_operator.cuh -- create_sparse_operator with an arbitrary
 * __host__ __device__ functor, for translation units compiled by nvcc
 * (included by aboria_gb/Aboria.h under __CUDACC__).
 *
 * The reference's KernelSparse (src/Kernels.h:692-751) calls the user's
 * closure f(dx, a, b) for every neighbour pair the radius search returns and
 * accumulates f * b_j in FP64.  Here the closure is f(dx, i, j) with dx the
 * Vector<double, D> separation x_j - x_i (periodic minimum image) and i, j the
 * row and column storage indices.  The operator is built once from the
 * library's FP64 radius search (abx_radius_query_csr: the same inclusive
 * |dx|^2 <= r^2 test) and keeps the neighbour lists on the device; each
 * K * b launches one kernel instantiated for F in the caller's translation
 * unit, one warp per row, FP64 evaluation and accumulation.  A functor that
 * returns Vector<double, BR> makes a block operator with BR rows per particle
 * (the reference's Eigen-block kernels, src/Kernels.h:692-718).  Memory is 8 B
 * per row plus 4 B per pair, so this path is meant for user closures at
 * moderate sizes; the built-in kernels (Aboria::kernels) run on the library's
 * tiled pair kernels without neighbour lists.
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

template <unsigned D> struct Domain {
  double width[D];
  int periodic[D];
};

// Rows of a functor's value: 1 for a double, BR for Vector<double, BR> (the
// reference's block operators, whose kernels return an Eigen BR x 1 block:
// row i of the operator becomes rows i*BR .. i*BR+BR-1).
template <typename R> struct BlockRows {
  static constexpr unsigned value = 1;
  static __host__ __device__ double get(const R &r, unsigned) { return r; }
};
template <unsigned BR> struct BlockRows<Vector<double, BR>> {
  static constexpr unsigned value = BR;
  static __host__ __device__ double get(const Vector<double, BR> &r, unsigned k) { return r[k]; }
};

template <unsigned D, typename F>
__global__ void functor_sparse_matvec(const int64_t *__restrict__ rowptr,
                                      const int32_t *__restrict__ cols,
                                      const double *__restrict__ rpos,
                                      const double *__restrict__ cpos, Domain<D> dom, F f,
                                      const double *__restrict__ b, double *__restrict__ c,
                                      int64_t nrows) {
  using R = decltype(f(Vector<double, D>(), int64_t(0), int64_t(0)));
  constexpr unsigned BR = BlockRows<R>::value;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nrows) return;
  const int64_t i = warp;
  double xi[D];
  for (unsigned d = 0; d < D; ++d) xi[d] = rpos[i * D + d];
  double acc[BR];
  for (unsigned k = 0; k < BR; ++k) acc[k] = 0.0;
  for (int64_t t = rowptr[i] + lane; t < rowptr[i + 1]; t += 32) {
    const int32_t j = cols[t];
    Vector<double, D> dx;
    for (unsigned d = 0; d < D; ++d) {
      double v = cpos[(int64_t)j * D + d] - xi[d];
      if (dom.periodic[d]) {
        const double w = dom.width[d];
        while (v > 0.5 * w) v -= w;
        while (v <= -0.5 * w) v += w;
      }
      dx[d] = v;
    }
    const R v = f(dx, i, (int64_t)j);
    for (unsigned k = 0; k < BR; ++k) acc[k] += BlockRows<R>::get(v, k) * b[j];
  }
  for (unsigned k = 0; k < BR; ++k) {
    double a = acc[k];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) c[i * BR + k] = a;
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

}  // namespace detail

/* The operator returned for a user functor; same K * b interface as
 * Aboria::Operator. */
template <unsigned D, typename F> class FunctorOperator {
  using R = decltype(std::declval<F>()(Vector<double, D>(), int64_t(0), int64_t(0)));

 public:
  static constexpr unsigned block_rows = detail::BlockRows<R>::value;

  template <typename RowP, typename ColP>
  FunctorOperator(const RowP &rows, const ColP &cols, double radius, F f)
      : nrows_(int64_t(rows.size())), ncols_(int64_t(cols.size())), f_(f) {
    static_assert(RowP::dimension == D && ColP::dimension == D, "dimension mismatch");
    if (!cols.searched()) {
      detail::check(ABX_ERR_STATE, "create_sparse_operator before init_neighbour_search");
      return;
    }
    for (unsigned d = 0; d < D; ++d) {
      dom_.width[d] = cols.get_max()[d] - cols.get_min()[d];
      dom_.periodic[d] = cols.get_periodic()[d] ? 1 : 0;
    }
    const double *q = nrows_ ? &rows.positions()[0][0] : nullptr;
    rowptr_.reset(new detail::DeviceArray<int64_t>(size_t(nrows_) + 1));
    // the library works on its context's (non-blocking) stream: wait for it
    // before the copies below, which use the legacy default stream
    abx_context *ctx = cols.context()->get();
    detail::check(abx_radius_query_csr(cols.handle(), nrows_, q, radius, rowptr_->ptr, nullptr, 0),
                  "create_sparse_operator: radius search");
    detail::check(abx_context_synchronize(ctx), "abx_context_synchronize");
    int64_t nnz = 0;
    detail::check_cuda(cudaMemcpy(&nnz, rowptr_->ptr + nrows_, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost),
                       "cudaMemcpy");
    cols_.reset(new detail::DeviceArray<int32_t>(size_t(nnz)));
    detail::check(abx_radius_query_csr(cols.handle(), nrows_, q, radius, rowptr_->ptr, cols_->ptr,
                                       nnz),
                  "create_sparse_operator: radius search");
    detail::check(abx_context_synchronize(ctx), "abx_context_synchronize");
    rpos_.reset(new detail::DeviceArray<double>(size_t(nrows_) * D));
    cpos_.reset(new detail::DeviceArray<double>(size_t(ncols_) * D));
    if (nrows_)
      detail::check_cuda(cudaMemcpy(rpos_->ptr, q, size_t(nrows_) * D * sizeof(double),
                                    cudaMemcpyHostToDevice),
                         "cudaMemcpy");
    if (ncols_)
      detail::check_cuda(cudaMemcpy(cpos_->ptr, &cols.positions()[0][0],
                                    size_t(ncols_) * D * sizeof(double), cudaMemcpyHostToDevice),
                         "cudaMemcpy");
    nnz_ = nnz;
  }

  int64_t rows() const { return nrows_ * block_rows; }
  int64_t cols() const { return ncols_; }
  /* stored pairs times the block size (the reference's assembled nnz) */
  int64_t nonzeros() const { return nnz_ * block_rows; }

  /* c = K * b with b and c in device memory, on the legacy default stream. */
  void apply_device(const double *b, double *c) const {
    if (nrows_ == 0) return;
    const int threads = 256;
    const int64_t blocks = (nrows_ * 32 + threads - 1) / threads;
    detail::functor_sparse_matvec<D, F><<<(unsigned)blocks, threads>>>(
        rowptr_->ptr, cols_->ptr, rpos_->ptr, cpos_->ptr, dom_, f_, b, c, nrows_);
    detail::check_cuda(cudaGetLastError(), "functor_sparse_matvec launch");
  }

  template <typename Vec> Vec operator*(const Vec &b) const {
    if (int64_t(b.size()) != ncols_) {
      detail::check(ABX_ERR_INVALID, "K*b: size of b does not match the operator's columns");
      return Vec();
    }
    Vec c(static_cast<size_t>(nrows_ * block_rows));
    detail::DeviceArray<double> db(static_cast<size_t>(ncols_)),
        dc(static_cast<size_t>(nrows_ * block_rows));
    if (ncols_)
      detail::check_cuda(cudaMemcpy(db.ptr, b.data(), size_t(ncols_) * sizeof(double),
                                    cudaMemcpyHostToDevice),
                         "cudaMemcpy");
    apply_device(db.ptr, dc.ptr);
    if (nrows_)
      detail::check_cuda(cudaMemcpy(c.data(), dc.ptr, size_t(nrows_ * block_rows) * sizeof(double),
                                    cudaMemcpyDeviceToHost),
                         "cudaMemcpy");
    return c;
  }

 private:
  int64_t nrows_, ncols_, nnz_ = 0;
  F f_;
  detail::Domain<D> dom_{};
  std::shared_ptr<detail::DeviceArray<int64_t>> rowptr_;
  std::shared_ptr<detail::DeviceArray<int32_t>> cols_;
  std::shared_ptr<detail::DeviceArray<double>> rpos_, cpos_;
};

/* create_sparse_operator(rows, cols, radius, f) with a __host__ __device__
 * functor f(dx, i, j) -> double (src/Operators.h:478-515). */
template <typename RowP, typename ColP, typename F,
          typename = typename std::enable_if<!std::is_same<
              typename std::decay<F>::type, abx_kernel>::value>::type>
FunctorOperator<RowP::dimension, F> create_sparse_operator(const RowP &row_particles,
                                                           const ColP &col_particles,
                                                           double radius, F f) {
  return FunctorOperator<RowP::dimension, F>(row_particles, col_particles, radius, f);
}

}  // namespace Aboria

#endif  // ABORIA_GB_FUNCTOR_OPERATOR_CUH_
