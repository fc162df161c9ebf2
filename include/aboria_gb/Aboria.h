/*
 * aboria_gb/Aboria.h -- C++ host layer over the abx C ABI with the names,
 * argument meanings and error behaviour of Aboria's hot-path API:
 *
 *   Particles<std::tuple<...>, D, Storage, SearchMethod>   src/Particles.h:108-112
 *     push_back, size, init_neighbour_search, update_positions, get<position>,
 *     get<id>
 *   CellListOrdered / HyperOctree (search-method tags)       src/CellListOrdered.h, src/OctTree.h
 *   euclidean_search(query, x, r[, transform])               src/Search.h:839-845,
 *     create_linear_transform, create_scale_transform         src/Transform.h
 *   create_sparse_operator / create_dense_operator /
 *   create_fmm_operator<N>                                   src/Operators.h:312-515
 *   K * b on any contiguous double vector (Eigen::VectorXd, std::vector<double>)
 *   SchwartzPreconditioner and an Eigen-shaped GMRES         src/Preconditioners.h:1121-1537,
 *                                                            tests/rbf_interpolation.h:360-370
 *
 * User variables.  ABORIA_VARIABLE(name, type, "name") declares a particle
 * variable (src/Variable.h); Particles<std::tuple<name, ...>, D> stores one
 * column per variable, reads and writes it with get<name>(particles)[i] or
 * get<name>(particle) on a value_type, and reorders it with the positions.
 *
 * Kernel functors.  The built-in closures of the reference's tests and
 * benchmarks are kernel descriptors (Aboria::kernels::*), evaluated by the
 * library's pair kernels.  Under nvcc (include/aboria_gb/functor_operator.cuh)
 * the operators also take the reference's closures as __host__ __device__
 * functors: create_sparse_operator(rows, cols, r, f(dx, a, b)) and its
 * variable-radius form create_sparse_operator(rows, cols, r(a), f(dx, a, b)),
 * create_dense_operator(rows, cols, f(a, b)), where a and b are particle
 * references read with get<position>/get<id>/get<variable> on the device;
 * their matvecs are matrix-free kernels instantiated in the caller's
 * translation unit over the library's cell list.  create_zero_operator and
 * create_block_operator<NI, NJ> compose any of these (src/Operators.h:519-548).
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

#include <algorithm>
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
/* position_d<D> (src/Variable.h): the reference's position variable type,
 * read and written like position. */
template <unsigned int D> struct position_d {};

/* ABORIA_VARIABLE(NAME, DATA_TYPE, NAME_STRING) (src/Variable.h): a particle
 * variable NAME holding one DATA_TYPE per particle. */
#define ABORIA_VARIABLE(NAME, DATA_TYPE, NAME_STRING)      \
  struct NAME {                                            \
    typedef DATA_TYPE value_type;                          \
    static const char *name() { return NAME_STRING; }      \
  };

namespace detail {
template <typename T> struct is_position : std::false_type {};
template <> struct is_position<position> : std::true_type {};
template <unsigned int D> struct is_position<position_d<D>> : std::true_type {};

// index of T in the pack (sizeof...(Vs) if absent)
template <typename T, typename... Vs> struct index_of;
template <typename T> struct index_of<T> : std::integral_constant<size_t, 0> {};
template <typename T, typename... Vs>
struct index_of<T, T, Vs...> : std::integral_constant<size_t, 0> {};
template <typename T, typename U, typename... Vs>
struct index_of<T, U, Vs...> : std::integral_constant<size_t, 1 + index_of<T, Vs...>::value> {};
}  // namespace detail

/* One particle by value (Particles::value_type): position, id and the
 * variables, read and written with get<...>(p). */
template <unsigned int D, typename... Vars> struct ParticleValue {
  Vector<double, D> pos;
  int64_t id_ = -1;
  std::tuple<typename Vars::value_type...> vars;
};

/* ----------------------------------------------------------- particles ---- */
/* A particle seen from a kernel: device pointers into the particle set's
 * columns and the particle's storage index (the reference's
 * Particles::const_reference, read with get<position>, get<id> and
 * get<variable>).  Built by the user-functor operators
 * (aboria_gb/functor_operator.cuh); valid inside their kernels. */
template <unsigned int D, typename... Vars> struct ParticleRef {
  const double *pos;  // SoA: pos[d * n + index]
  int64_t n;
  const int64_t *ids;
  const void *vars[sizeof...(Vars) > 0 ? sizeof...(Vars) : 1];
  int64_t index;
};

template <typename Variables, unsigned int D = 3, typename Storage = void,
          typename SearchMethod = CellListOrdered>
class Particles;

template <typename... Vars, unsigned int D, typename Storage, typename SearchMethod>
class Particles<std::tuple<Vars...>, D, Storage, SearchMethod> {
  static_assert(D >= 1 && D <= 3, "the GPU path supports 1 to 3 dimensions");

 public:
  typedef void particles_tag;
  typedef Vector<double, D> double_d;
  typedef Vector<bool, D> bool_d;
  typedef ParticleValue<D, Vars...> value_type;
  typedef ParticleRef<D, Vars...> const_reference;
  typedef ParticleRef<D, Vars...> reference;
  typedef std::tuple<Vars...> variables_type;
  typedef SearchMethod search_method;
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
    resize_vars(n);
    next_id_ = int64_t(n);
    dirty_ = true;
  }

  size_t size() const { return pos_.size(); }

  /* push_back(particle) / push_back(position): appended with the next id;
   * takes effect on the device at the next init_neighbour_search /
   * update_positions. */
  void push_back(const value_type &v) {
    if (searched_ && !dirty_) {
      // a searchable set is updated at once (src/Particles.h:264-283)
      const std::vector<int64_t> before = ids_;
      int64_t nid = 0;
      detail::check(abx_particles_push_back(h_.get(), 1, v.pos.data(), &nid), "push_back");
      ids_.push_back(nid);
      next_id_ = nid + 1;
      push_vars(v.vars, std::index_sequence_for<Vars...>());
      std::vector<int64_t> with_new = before;
      with_new.push_back(nid);
      download(with_new);
      return;
    }
    pos_.push_back(v.pos);
    ids_.push_back(next_id_++);
    push_vars(v.vars, std::index_sequence_for<Vars...>());
    dirty_ = true;
    ++version_;
  }

  /* erase(i) / erase(first, last) (src/Particles.h:361-389): the particles at
   * storage positions [first, last) are dropped; a searchable set is updated
   * at once. */
  void erase(size_t first, size_t last) {
    if (first >= last) return;
    if (searched_ && !dirty_) {
      std::vector<int64_t> before = ids_;
      detail::check(abx_particles_erase(h_.get(), int64_t(first), int64_t(last)), "erase");
      download(before);
      return;
    }
    pos_.erase(pos_.begin() + first, pos_.begin() + last);
    ids_.erase(ids_.begin() + first, ids_.begin() + last);
    apply_vars([&](auto &col) { col.erase(col.begin() + first, col.begin() + last); });
    dirty_ = true;
    ++version_;
  }
  void erase(size_t i) { erase(i, i + 1); }

  /* Find-by-id (src/NeighbourSearchBase.h:276-321): the storage position of
   * the particle with this id, or size() when there is none (the reference
   * returns end()). */
  size_t find(int64_t particle_id) {
    upload();
    int64_t idx = -1;
    detail::check(abx_particles_find_ids(h_.get(), 1, &particle_id, &idx), "find");
    return idx < 0 ? size() : size_t(idx);
  }
  void push_back(const double_d &x) {
    value_type v;
    v.pos = x;
    push_back(v);
  }

  std::vector<double_d> &positions() { dirty_ = true; ++version_; return pos_; }
  const std::vector<double_d> &positions() const { return pos_; }
  const std::vector<int64_t> &ids() const { return ids_; }
  /* the host column of variable V (get<V>(particles)) */
  template <typename V> std::vector<typename V::value_type> &variable() {
    ++version_;
    return std::get<detail::index_of<V, Vars...>::value>(vars_);
  }
  template <typename V> const std::vector<typename V::value_type> &variable() const {
    return std::get<detail::index_of<V, Vars...>::value>(vars_);
  }
  const std::tuple<std::vector<typename Vars::value_type>...> &variables() const { return vars_; }

  /* init_neighbour_search(low, high, periodic, n_particles_in_leaf)
   * (src/Particles.h:445-456): uploads the particles, builds the search
   * structure of SearchMethod and reorders the storage, variables included. */
  void init_neighbour_search(const double_d &low, const double_d &high, const bool_d &periodic,
                             double n_particles_in_leaf = 10) {
    const std::vector<int64_t> before = ids_;
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
    download(before);
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
    const std::vector<int64_t> before = ids_;
    detail::check(abx_particles_set_positions(h_.get(), &pos_[0][0]), "set_positions");
    detail::check(abx_particles_update_positions(h_.get()), "update_positions");
    download(before);
  }

  abx_particles *handle() const { return h_.get(); }
  const std::shared_ptr<detail::Context> &context() const { return ctx_; }
  bool searched() const { return searched_; }
  const double_d &get_min() const { return low_; }
  const double_d &get_max() const { return high_; }
  const bool_d &get_periodic() const { return periodic_; }
  /* changes with every change of the host storage (the user-functor
   * operators re-upload the variable columns when it moved) */
  uint64_t version() const { return version_; }
  /* device copies of the variable columns, owned here, filled by the
   * user-functor operators */
  std::shared_ptr<void> &device_cache() const { return device_cache_; }

 private:
  template <size_t... I>
  void push_vars(const std::tuple<typename Vars::value_type...> &v, std::index_sequence<I...>) {
    int dummy[] = {0, (std::get<I>(vars_).push_back(std::get<I>(v)), 0)...};
    (void)dummy;
  }
  void resize_vars(size_t n) {
    apply_vars([n](auto &col) { col.resize(n); });
  }
  template <typename Fn> void apply_vars(Fn fn) {
    apply_vars_impl(fn, std::index_sequence_for<Vars...>());
  }
  template <typename Fn, size_t... I> void apply_vars_impl(Fn fn, std::index_sequence<I...>) {
    int dummy[] = {0, (fn(std::get<I>(vars_)), 0)...};
    (void)dummy;
  }
  void upload() {
    if (!dirty_) return;
    const int64_t n = int64_t(pos_.size());
    detail::check(abx_particles_set(h_.get(), n, n ? &pos_[0][0] : nullptr,
                                    n ? ids_.data() : nullptr),
                  "abx_particles_set");
    dirty_ = false;
  }
  /* positions and ids in the new storage order; the variables follow the
   * particles through their ids (`before` = the ids in the previous order) */
  void download(const std::vector<int64_t> &before) {
    const int64_t n = abx_particles_size(h_.get());
    pos_.resize(size_t(n));
    ids_.resize(size_t(n));
    if (n) {
      detail::check(abx_particles_get_positions(h_.get(), &pos_[0][0]), "get_positions");
      detail::check(abx_particles_get_ids(h_.get(), ids_.data()), "get_ids");
    }
    if (sizeof...(Vars) > 0) {
      std::vector<std::pair<int64_t, size_t>> by_id(before.size());
      for (size_t k = 0; k < before.size(); ++k) by_id[k] = {before[k], k};
      std::sort(by_id.begin(), by_id.end());
      std::vector<size_t> src(static_cast<size_t>(n));
      for (size_t k = 0; k < size_t(n); ++k) {
        auto it = std::lower_bound(by_id.begin(), by_id.end(), std::make_pair(ids_[k], size_t(0)));
        src[k] = it->second;
      }
      apply_vars([&src](auto &col) {
        typename std::decay<decltype(col)>::type out(src.size());
        for (size_t k = 0; k < src.size(); ++k) out[k] = col[src[k]];
        col.swap(out);
      });
    }
    dirty_ = false;
    ++version_;
  }

  static_assert(sizeof(Vector<double, D>) == D * sizeof(double), "packed positions");
  std::shared_ptr<detail::Context> ctx_;
  std::shared_ptr<abx_particles> h_;
  std::vector<double_d> pos_;
  std::vector<int64_t> ids_;
  std::tuple<std::vector<typename Vars::value_type>...> vars_;
  double_d low_, high_;
  bool_d periodic_;
  int64_t next_id_ = 0;
  bool dirty_ = true;
  bool searched_ = false;
  uint64_t version_ = 0;
  mutable std::shared_ptr<void> device_cache_;
};

namespace detail {
template <typename Tag, typename Enable = void> struct getter {
  template <typename P> static decltype(auto) get(P &p) { return p.template variable<Tag>(); }
};
template <typename Tag> struct getter<Tag, typename std::enable_if<is_position<Tag>::value>::type> {
  template <typename P> static decltype(auto) get(P &p) { return p.positions(); }
};
template <> struct getter<id> {
  template <typename P> static const std::vector<int64_t> &get(P &p) { return p.ids(); }
};

template <typename Tag, typename Enable = void> struct value_getter {
  template <unsigned D, typename... V> static auto &get(ParticleValue<D, V...> &p) {
    return std::get<index_of<Tag, V...>::value>(p.vars);
  }
  template <unsigned D, typename... V> static const auto &get(const ParticleValue<D, V...> &p) {
    return std::get<index_of<Tag, V...>::value>(p.vars);
  }
};
template <typename Tag>
struct value_getter<Tag, typename std::enable_if<is_position<Tag>::value>::type> {
  template <typename P> static auto &get(P &p) { return p.pos; }
};
template <> struct value_getter<id> {
  template <typename P> static auto &get(P &p) { return p.id_; }
};

template <typename Tag, typename Enable = void> struct ref_getter {
  template <unsigned D, typename... V>
  ABORIA_GB_HD static typename Tag::value_type get(const ParticleRef<D, V...> &r) {
    return static_cast<const typename Tag::value_type *>(r.vars[index_of<Tag, V...>::value])[r.index];
  }
};
template <typename Tag>
struct ref_getter<Tag, typename std::enable_if<is_position<Tag>::value>::type> {
  template <unsigned D, typename... V>
  ABORIA_GB_HD static Vector<double, D> get(const ParticleRef<D, V...> &r) {
    Vector<double, D> x;
    for (unsigned d = 0; d < D; ++d) x[d] = r.pos[d * r.n + r.index];
    return x;
  }
};
template <> struct ref_getter<id> {
  template <unsigned D, typename... V>
  ABORIA_GB_HD static int64_t get(const ParticleRef<D, V...> &r) { return r.ids[r.index]; }
};
}  // namespace detail

/* get<position>(particles)[i] / get<id>(particles)[i] / get<var>(particles)[i]
 * (src/Get.h): the host columns of a particle set. */
template <typename Tag, typename P,
          typename = typename std::decay<P>::type::particles_tag>
decltype(auto) get(P &p) {
  return detail::getter<Tag>::get(p);
}
/* get<...>(value): a particle held by value (Particles::value_type). */
template <typename Tag, unsigned int D, typename... V> auto &get(ParticleValue<D, V...> &p) {
  return detail::value_getter<Tag>::get(p);
}
template <typename Tag, unsigned int D, typename... V>
const auto &get(const ParticleValue<D, V...> &p) {
  return detail::value_getter<Tag>::get(p);
}
/* get<...>(a) on a particle reference inside a user functor (device code). */
template <typename Tag, unsigned int D, typename... V>
ABORIA_GB_HD auto get(const ParticleRef<D, V...> &r) {
  return detail::ref_getter<Tag>::get(r);
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
 * particle (and periodic image) with |x_j - x|^2 <= r^2 in FP64, with dx the
 * separation x_j - (x + image*L) of the image the search accepted
 * (src/Search.h:188-190, 443).  One query per call; many queries belong in
 * abx_radius_count / abx_radius_query_csr. */
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
  const size_t nnz = static_cast<size_t>(rowptr[1]);
  std::vector<int32_t> cols(nnz);
  std::vector<double> dx(nnz * D);
  if (nnz)
    detail::check(abx_radius_query_csr_dx(particles.handle(), 1, x.data(), r, rowptr, cols.data(),
                                          dx.data(), rowptr[1]),
                  "euclidean_search");
  for (size_t k = 0; k < nnz; ++k) {
    SearchResult<D> s;
    s.index = cols[k];
    for (unsigned d = 0; d < D; ++d) s.dx[d] = dx[k * D + d];
    out.push_back(s);
  }
  return out;
}

/* Linear coordinate transforms for the searches (src/Transform.h): the
 * transform's D x D matrix, column k = f(e_k) of the user's linear map f
 * (exact for the reference's maps whose coefficients multiply single
 * coordinates: the matrix form adds the other coordinates times zero). */
template <unsigned int D> struct LinearTransformMatrix {
  double m[D * D];  // row-major
};
template <unsigned int D, typename F> LinearTransformMatrix<D> create_linear_transform(const F &f) {
  LinearTransformMatrix<D> t;
  for (unsigned k = 0; k < D; ++k) {
    Vector<double, D> e;
    e[k] = 1.0;
    const Vector<double, D> col = f(e);
    for (unsigned i = 0; i < D; ++i) t.m[i * D + k] = col[i];
  }
  return t;
}
/* create_scale_transform(s): x_d -> s_d x_d */
template <unsigned int D> LinearTransformMatrix<D> create_scale_transform(const Vector<double, D> &s) {
  LinearTransformMatrix<D> t;
  for (unsigned i = 0; i < D * D; ++i) t.m[i] = 0.0;
  for (unsigned i = 0; i < D; ++i) t.m[i * D + i] = s[i];
  return t;
}

/* euclidean_search(query, x, r, transform) (src/Search.h:839-845 with a
 * LinearTransform): the neighbours with |T dx| <= r; dx is returned
 * transformed, as the reference's dx() is (abx_radius_query_csr_transform). */
template <typename P>
std::vector<SearchResult<P::dimension>> euclidean_search(
    const P &particles, const typename P::double_d &x, double r,
    const LinearTransformMatrix<P::dimension> &transform) {
  constexpr unsigned D = P::dimension;
  std::vector<SearchResult<D>> out;
  if (!particles.searched()) {
    detail::check(ABX_ERR_STATE, "euclidean_search before init_neighbour_search");
    return out;
  }
  int64_t rowptr[2] = {0, 0};
  detail::check(abx_radius_query_csr_transform(particles.handle(), 1, x.data(), r, transform.m,
                                               rowptr, nullptr, nullptr, 0),
                "euclidean_search");
  const size_t nnz = static_cast<size_t>(rowptr[1]);
  std::vector<int32_t> cols(nnz);
  std::vector<double> dx(nnz * D);
  if (nnz)
    detail::check(abx_radius_query_csr_transform(particles.handle(), 1, x.data(), r, transform.m,
                                                 rowptr, cols.data(), dx.data(), rowptr[1]),
                  "euclidean_search");
  for (size_t k = 0; k < nnz; ++k) {
    SearchResult<D> s;
    s.index = cols[k];
    for (unsigned d = 0; d < D; ++d) s.dx[d] = dx[k * D + d];
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

/* create_zero_operator(rows, cols) (src/Operators.h:519-537): the rows x cols
 * zero operator, a placeholder block of create_block_operator. */
class ZeroOperator {
 public:
  ZeroOperator(int64_t r, int64_t c) : r_(r), c_(c) {}
  int64_t rows() const { return r_; }
  int64_t cols() const { return c_; }
  void apply(const double *, double *c) const {
    for (int64_t i = 0; i < r_; ++i) c[i] = 0.0;
  }
  template <typename Vec> Vec operator*(const Vec &b) const {
    if (int64_t(b.size()) != c_) {
      detail::check(ABX_ERR_INVALID, "K*b: size of b does not match the operator's columns");
      return Vec();
    }
    Vec c(static_cast<size_t>(r_));
    apply(b.data(), c.data());
    return c;
  }

 private:
  int64_t r_, c_;
};

template <typename RowP, typename ColP>
ZeroOperator create_zero_operator(const RowP &row_particles, const ColP &col_particles) {
  return ZeroOperator(int64_t(row_particles.size()), int64_t(col_particles.size()));
}

/* create_block_operator<NI, NJ>(K_00, K_01, ..., K_(NI-1)(NJ-1))
 * (src/Operators.h:539-548, MatrixReplacement<NI, NJ, ...>): an NI x NJ
 * matrix of operators given row by row; block (i, j) spans the rows of block
 * (i, 0) and the columns of block (0, j) (start_row/start_col,
 * src/Operators.h:219-234), and K * b sums K_ij b_j into each block row. */
template <unsigned int NI, unsigned int NJ, typename... Ops> class BlockOperator {
  static_assert(sizeof...(Ops) == NI * NJ, "create_block_operator<NI, NJ> takes NI*NJ operators");

 public:
  explicit BlockOperator(const Ops &...ops) : ops_(ops...) {}

  int64_t rows() const {
    int64_t n = 0;
    for (unsigned i = 0; i < NI; ++i) n += block_rows(i);
    return n;
  }
  int64_t cols() const {
    int64_t n = 0;
    for (unsigned j = 0; j < NJ; ++j) n += block_cols(j);
    return n;
  }

  void apply(const double *b, double *c) const {
    int64_t r0 = 0;
    for (unsigned i = 0; i < NI; ++i) {
      const int64_t nr = block_rows(i);
      for (int64_t k = 0; k < nr; ++k) c[r0 + k] = 0.0;
      std::vector<double> tmp(static_cast<size_t>(nr));
      int64_t c0 = 0;
      for (unsigned j = 0; j < NJ; ++j) {
        for_block(i * NJ + j, [&](const auto &op) {
          if (nr > 0) op.apply(b + c0, tmp.data());
        });
        for (int64_t k = 0; k < nr; ++k) c[r0 + k] += tmp[size_t(k)];
        c0 += block_cols(j);
      }
      r0 += nr;
    }
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

 private:
  template <typename Fn> void for_block(unsigned k, Fn fn) const {
    for_block_impl(k, fn, std::index_sequence_for<Ops...>());
  }
  template <typename Fn, size_t... I>
  void for_block_impl(unsigned k, Fn fn, std::index_sequence<I...>) const {
    int dummy[] = {0, (I == k ? (fn(std::get<I>(ops_)), 0) : 0)...};
    (void)dummy;
  }
  int64_t block_rows(unsigned i) const {
    int64_t n = 0;
    for_block(i * NJ, [&](const auto &op) { n = op.rows(); });
    return n;
  }
  int64_t block_cols(unsigned j) const {
    int64_t n = 0;
    for_block(j, [&](const auto &op) { n = op.cols(); });
    return n;
  }
  std::tuple<Ops...> ops_;
};

template <unsigned int NI, unsigned int NJ, typename... Ops>
BlockOperator<NI, NJ, Ops...> create_block_operator(const Ops &...ops) {
  return BlockOperator<NI, NJ, Ops...>(ops...);
}

/* create_h2_operator(rows, cols, order, kernel, eta) (src/Operators.h:440-447):
 * the black-box H2 operator with a runtime Chebyshev order and the
 * admissibility parameter eta on the HyperOctree of one particle set. */
template <typename RowP, typename ColP>
Operator create_h2_operator(const RowP &row_particles, const ColP &col_particles, int order,
                            const abx_kernel &kernel, double eta = 1.0) {
  if (row_particles.handle() != col_particles.handle()) {
    detail::check(ABX_ERR_INVALID, "create_h2_operator: rows and cols must be one particle set");
    return Operator();
  }
  abx_operator *h = nullptr;
  detail::check(abx_create_h2_operator(row_particles.handle(), &kernel, order, eta, &h),
                "create_h2_operator");
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
#include "symbolic.cuh"
#endif

#endif  // ABORIA_GB_ABORIA_H_
