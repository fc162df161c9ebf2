/*
 * aboria_gb/symbolic.cuh -- the reference's Level-3 symbolic neighbour sums
 * (src/Symbolic.h, src/Functions.h), for translation units compiled by nvcc,
 * lowered onto the matrix-free user-functor kernels of functor_operator.cuh:
 *
 *   Symbol<position> p;  Symbol<a_var> a;          variables      src/Symbolic.h
 *   Label<0, P> i(particles);  Label<1, Q> j(others);  labels
 *   auto dx = create_dx(i, j);                     x_j - x_i of the accepted image
 *   Accumulate<std::plus<T>> sum;                  the reduction
 *   a[i] = sum(j, norm(dx) < r, expr);             sparse: a neighbour search of radius r
 *   a[i] += sum(j, true, expr);                    dense: every j
 *
 * An expression is built from dx, norm(...), the variables at i or j
 * (s[i], s[j]), literals, + - * / (scalars and Vector<double, N>), the
 * comparisons < <= > >= and if_else(c, x, y) (src/Functions.h).  A sum whose
 * condition is `norm(dx) < r` (r a number) searches the column particles'
 * CellListOrdered grid with radius r -- the reference's search is inclusive
 * (!(|dx|^2 > r^2), src/Search.h:438-465) and the condition is then
 * evaluated on every candidate, so a pair exactly at r is not summed; any
 * other condition visits every j and evaluates the condition.  The label j
 * runs over all particles of its set, i itself included (dx = 0).  The
 * assignment runs one kernel instantiated for the expression (the sum over
 * j of cond ? expr : 0, one warp per row i for the sparse form) and writes
 * the host column of the assigned variable.  A value is a double or a
 * Vector<double, N>; integer accumulations are carried in double.
 *
 * eval(sum(i, x)) sums over the row particles a per-particle value x, itself
 * a sum over j or an expression of i.  AccumulateWithinDistance<std::plus<T>,
 * LNorm>(r) sums over the neighbours within r in the 2-, 1- or inf-norm.
 *
 * Not covered: a sum inside an arithmetic expression, sums over labels other
 * than the row label and the column label, min/max accumulations, the
 * reference's geometry functions beyond norm.
 */
#ifndef ABORIA_GB_SYMBOLIC_CUH_
#define ABORIA_GB_SYMBOLIC_CUH_

#include <cmath>
#include <functional>
#include <type_traits>

namespace Aboria {

namespace sym {

// ---- value arithmetic: doubles and Vector<double, N>
template <typename T> struct is_vec : std::false_type {};
template <unsigned N> struct is_vec<Vector<double, N>> : std::true_type {};

template <typename T> ABORIA_GB_HD inline double as_double(const T &v) { return double(v); }

struct OpAdd {
  ABORIA_GB_HD static double f(double a, double b) { return a + b; }
};
struct OpSub {
  ABORIA_GB_HD static double f(double a, double b) { return a - b; }
};
struct OpMul {
  ABORIA_GB_HD static double f(double a, double b) { return a * b; }
};
struct OpDiv {
  ABORIA_GB_HD static double f(double a, double b) { return a / b; }
};

template <typename Op> ABORIA_GB_HD inline double apply(double a, double b) { return Op::f(a, b); }
template <typename Op, unsigned N>
ABORIA_GB_HD inline Vector<double, N> apply(const Vector<double, N> &a, const Vector<double, N> &b) {
  Vector<double, N> r;
  for (unsigned k = 0; k < N; ++k) r[k] = Op::f(a[k], b[k]);
  return r;
}
template <typename Op, unsigned N>
ABORIA_GB_HD inline Vector<double, N> apply(const Vector<double, N> &a, double b) {
  Vector<double, N> r;
  for (unsigned k = 0; k < N; ++k) r[k] = Op::f(a[k], b);
  return r;
}
template <typename Op, unsigned N>
ABORIA_GB_HD inline Vector<double, N> apply(double a, const Vector<double, N> &b) {
  Vector<double, N> r;
  for (unsigned k = 0; k < N; ++k) r[k] = Op::f(a, b[k]);
  return r;
}

ABORIA_GB_HD inline double norm_of(double v) { return v < 0 ? -v : v; }
template <unsigned N> ABORIA_GB_HD inline double norm_of(const Vector<double, N> &v) {
  return sqrt(v.squaredNorm());
}

// ---- expression nodes: E::eval(dx, a, b) with a the row particle, b the column one
struct ExprTag {};

template <typename T> struct Lit : ExprTag {
  T v;
  template <typename V, typename A, typename B>
  ABORIA_GB_HD T eval(const V &, const A &, const B &) const {
    return v;
  }
};

struct Dx : ExprTag {
  template <typename V, typename A, typename B>
  ABORIA_GB_HD V eval(const V &dx, const A &, const B &) const {
    return dx;
  }
};

template <typename Tag, int L> struct VarAt : ExprTag {
  template <typename V, typename A, typename B>
  ABORIA_GB_HD auto eval(const V &, const A &a, const B &b) const {
    if constexpr (L == 0)
      return detail::ref_getter<Tag>::get(a);
    else
      return detail::ref_getter<Tag>::get(b);
  }
};

template <typename E> struct Norm : ExprTag {
  E e;
  template <typename V, typename A, typename B>
  ABORIA_GB_HD double eval(const V &dx, const A &a, const B &b) const {
    return norm_of(e.eval(dx, a, b));
  }
};

template <typename Op, typename L, typename R> struct Bin : ExprTag {
  L l;
  R r;
  template <typename V, typename A, typename B>
  ABORIA_GB_HD auto eval(const V &dx, const A &a, const B &b) const {
    return apply<Op>(l.eval(dx, a, b), r.eval(dx, a, b));
  }
};

struct CmpLt {
  ABORIA_GB_HD static bool f(double a, double b) { return a < b; }
};
struct CmpLe {
  ABORIA_GB_HD static bool f(double a, double b) { return a <= b; }
};
struct CmpGt {
  ABORIA_GB_HD static bool f(double a, double b) { return a > b; }
};
struct CmpGe {
  ABORIA_GB_HD static bool f(double a, double b) { return a >= b; }
};
struct CmpEq {
  ABORIA_GB_HD static bool f(double a, double b) { return a == b; }
};

template <typename Op, typename L, typename R> struct Cmp : ExprTag {
  L l;
  R r;
  template <typename V, typename A, typename B>
  ABORIA_GB_HD bool eval(const V &dx, const A &a, const B &b) const {
    return Op::f(as_double(l.eval(dx, a, b)), as_double(r.eval(dx, a, b)));
  }
};

template <typename C, typename X, typename Y> struct IfElse : ExprTag {
  C c;
  X x;
  Y y;
  template <typename V, typename A, typename B>
  ABORIA_GB_HD auto eval(const V &dx, const A &a, const B &b) const {
    typedef decltype(x.eval(dx, a, b)) TX;
    typedef decltype(y.eval(dx, a, b)) TY;
    typedef typename std::conditional<is_vec<TX>::value, TX, TY>::type T;
    if (c.eval(dx, a, b)) return T(x.eval(dx, a, b));
    return T(y.eval(dx, a, b));
  }
};

// literals and expressions alike
template <typename T> struct is_expr : std::is_base_of<ExprTag, T> {};
template <typename T, typename = void> struct as_expr {
  typedef Lit<T> type;
  static type make(const T &v) { return type{{}, v}; }
};
template <typename T> struct as_expr<T, typename std::enable_if<is_expr<T>::value>::type> {
  typedef T type;
  static const T &make(const T &e) { return e; }
};
template <typename T> using expr_t = typename as_expr<typename std::decay<T>::type>::type;
template <typename T> expr_t<T> make_expr(const T &v) {
  return as_expr<typename std::decay<T>::type>::make(v);
}

template <typename A, typename B>
using enable_bin = typename std::enable_if<is_expr<A>::value || is_expr<B>::value>::type;

template <typename A, typename B, typename = enable_bin<A, B>>
Bin<OpAdd, expr_t<A>, expr_t<B>> operator+(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Bin<OpSub, expr_t<A>, expr_t<B>> operator-(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Bin<OpMul, expr_t<A>, expr_t<B>> operator*(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Bin<OpDiv, expr_t<A>, expr_t<B>> operator/(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Cmp<CmpLt, expr_t<A>, expr_t<B>> operator<(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Cmp<CmpLe, expr_t<A>, expr_t<B>> operator<=(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Cmp<CmpGt, expr_t<A>, expr_t<B>> operator>(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Cmp<CmpGe, expr_t<A>, expr_t<B>> operator>=(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}
template <typename A, typename B, typename = enable_bin<A, B>>
Cmp<CmpEq, expr_t<A>, expr_t<B>> operator==(const A &a, const B &b) {
  return {{}, make_expr(a), make_expr(b)};
}

// the condition `norm(dx) < r` (r a number) fixes the search radius
template <typename C> struct radius_of {
  static constexpr bool sparse = false;
  static double get(const C &) { return 0.0; }
};
template <> struct radius_of<Cmp<CmpLt, Norm<Dx>, Lit<double>>> {
  static constexpr bool sparse = true;
  static double get(const Cmp<CmpLt, Norm<Dx>, Lit<double>> &c) { return c.r.v; }
};
template <> struct radius_of<Cmp<CmpLt, Norm<Dx>, Lit<int>>> {
  static constexpr bool sparse = true;
  static double get(const Cmp<CmpLt, Norm<Dx>, Lit<int>> &c) { return double(c.r.v); }
};
template <> struct radius_of<Cmp<CmpLe, Norm<Dx>, Lit<double>>> {
  static constexpr bool sparse = true;
  static double get(const Cmp<CmpLe, Norm<Dx>, Lit<double>> &c) { return c.r.v; }
};

// The pair functor handed to the user-functor kernels: cond ? value : 0 in
// the accumulation type T.
template <typename T, typename C, typename E> struct PairTerm {
  C c;
  E e;
  template <typename V, typename A, typename B>
  ABORIA_GB_HD T operator()(const V &dx, const A &a, const B &b) const {
    if (!c.eval(dx, a, b)) return T();
    return T(e.eval(dx, a, b));
  }
  // dense form f(a, b): dx = x_b - x_a without periodic images
  template <typename A, typename B> ABORIA_GB_HD T operator()(const A &a, const B &b) const {
    const auto xa = detail::ref_getter<position>::get(a);
    const auto xb = detail::ref_getter<position>::get(b);
    typename std::decay<decltype(xa)>::type dx;
    for (unsigned d = 0; d < sizeof(xa) / sizeof(double); ++d) dx[d] = xb[d] - xa[d];
    return (*this)(dx, a, b);
  }
};

template <typename T> struct acc_value {
  typedef double type;
};
template <unsigned N> struct acc_value<Vector<double, N>> {
  typedef Vector<double, N> type;
};

// sum over the column label j: within = true searches radius r (the
// reference's AccumulateWithinDistance), else the condition decides
template <typename P, typename T, typename C, typename E> struct Sum {
  const P *cols;
  C c;
  E e;
  bool within;
  double r;
  int lnorm;  // within: the search norm (2, 1 or -1)
};

// sum over the row label i of a per-particle value (a Sum over j or an
// expression of i), for eval(...)
template <typename P, typename T, typename C, typename X> struct SumAll {
  const P *rows;
  C c;
  X x;
};

// A particle reference to the host columns (positions copied to SoA), for
// the univariate assignments evaluated on the host.
template <typename P> struct HostRef {
  std::vector<double> soa;
  std::vector<const void *> vars;
  typename P::const_reference ref;
  explicit HostRef(const P &p) {
    constexpr unsigned D = P::dimension;
    const size_t n = p.size();
    soa.resize(n * D);
    for (size_t i = 0; i < n; ++i)
      for (unsigned d = 0; d < D; ++d) soa[d * n + i] = p.positions()[i][d];
    ref = typename P::const_reference{};
    ref.pos = soa.data();
    ref.n = int64_t(n);
    ref.ids = p.ids().data();
    size_t k = 0;
    std::apply([&](const auto &...col) {
      int dummy[] = {0, (ref.vars[k++] = static_cast<const void *>(col.data()), 0)...};
      (void)dummy;
    }, p.variables());
  }
};

}  // namespace sym

/* Label<L, P> (src/Symbolic.h): label 0 is the row (assigned) particle set,
 * label 1 the particle set summed over. */
template <int L, typename P> struct Label : sym::ExprTag {
  const P *p;
  explicit Label(const P &particles) : p(&particles) {}
};

/* create_dx(i, j): x_j - x_i (src/Symbolic.h) */
template <typename P, typename Q> sym::Dx create_dx(const Label<0, P> &, const Label<1, Q> &) {
  return {};
}

/* norm(e) (src/Functions.h) */
template <typename E, typename = typename std::enable_if<sym::is_expr<E>::value>::type>
sym::Norm<E> norm(const E &e) {
  return {{}, e};
}

/* if_else(cond, a, b) (src/Functions.h) */
template <typename C, typename X, typename Y>
sym::IfElse<sym::expr_t<C>, sym::expr_t<X>, sym::expr_t<Y>> if_else(const C &c, const X &x,
                                                                     const Y &y) {
  return {{}, sym::make_expr(c), sym::make_expr(x), sym::make_expr(y)};
}

/* Accumulate<std::plus<T>> (src/Symbolic.h): sum(j, cond, expr). */
namespace sym {
template <typename T> struct is_sum : std::false_type {};
template <typename P, typename T, typename C, typename E>
struct is_sum<Sum<P, T, C, E>> : std::true_type {};

// sum over j for every row particle: n x BR values (BR = 1 for a double)
template <int NORM, typename P, typename Q, typename F>
void run_sparse(const P &rows, const Q &cols, double r, const F &f, const double *ones, double *c) {
  const FunctorOperator<P, Q, F, detail::ConstRadius, false, NORM> op(rows, cols,
                                                                     detail::ConstRadius{r}, f);
  op.apply(ones, c);
}
template <typename P, typename Q, typename T, typename C, typename E>
std::vector<double> sum_values(const P &rows, const Sum<Q, T, C, E> &s) {
  typedef PairTerm<T, C, E> F;
  typedef radius_of<C> RO;
  const F f{s.c, s.e};
  const size_t n = rows.size(), nc = s.cols->size();
  constexpr unsigned BR = detail::BlockRows<T>::value;
  std::vector<double> c(n * BR, 0.0);
  if (n == 0 || nc == 0) return c;
  std::vector<double> ones(nc, 1.0);
  if (s.within || RO::sparse) {
    const double r = s.within ? s.r : RO::get(s.c);
    if (s.within && s.lnorm == 1)
      run_sparse<1>(rows, *s.cols, r, f, ones.data(), c.data());
    else if (s.within && s.lnorm == -1)
      run_sparse<-1>(rows, *s.cols, r, f, ones.data(), c.data());
    else
      run_sparse<2>(rows, *s.cols, r, f, ones.data(), c.data());
  } else {
    const auto op = create_dense_operator(rows, *s.cols, f);
    op.apply(ones.data(), c.data());
  }
  return c;
}
}  // namespace sym

/* Accumulate<std::plus<T>> (src/Symbolic.h): sum(j, cond, expr) or
 * sum(j, expr) over the column label; sum(i, expr) / sum(i, cond, expr)
 * over the row label, evaluated with eval(...). */
template <typename Functor> struct Accumulate;
template <typename T> struct Accumulate<std::plus<T>> {
  typedef typename sym::acc_value<T>::type value_type;
  template <typename Q, typename C, typename E>
  sym::Sum<Q, value_type, sym::expr_t<C>, sym::expr_t<E>> operator()(const Label<1, Q> &j,
                                                                     const C &cond,
                                                                     const E &e) const {
    return {j.p, sym::make_expr(cond), sym::make_expr(e), false, 0.0, 2};
  }
  template <typename Q, typename E>
  sym::Sum<Q, value_type, sym::Lit<bool>, sym::expr_t<E>> operator()(const Label<1, Q> &j,
                                                                     const E &e) const {
    return {j.p, sym::Lit<bool>{{}, true}, sym::make_expr(e), false, 0.0, 2};
  }
  template <typename P, typename C, typename X>
  sym::SumAll<P, value_type, sym::expr_t<C>, X> operator()(const Label<0, P> &i, const C &cond,
                                                            const X &x) const {
    return {i.p, sym::make_expr(cond), x};
  }
  template <typename P, typename X>
  sym::SumAll<P, value_type, sym::Lit<bool>, X> operator()(const Label<0, P> &i,
                                                            const X &x) const {
    return {i.p, sym::Lit<bool>{{}, true}, x};
  }
};

/* AccumulateWithinDistance<std::plus<T>, LNorm>(r) (src/Symbolic.h):
 * sum(j, expr) over the neighbours found by a search of radius r in the
 * LNorm norm (2 euclidean, 1 manhattan, -1 chebyshev; inclusive). */
template <typename Functor, int LNorm = 2> struct AccumulateWithinDistance;
template <typename T, int LNorm> struct AccumulateWithinDistance<std::plus<T>, LNorm> {
  static_assert(LNorm == 2 || LNorm == 1 || LNorm == -1, "norm 2, 1 or -1");
  typedef typename sym::acc_value<T>::type value_type;
  double radius;
  explicit AccumulateWithinDistance(double r) : radius(r) {}
  template <typename Q, typename E>
  sym::Sum<Q, value_type, sym::Lit<bool>, sym::expr_t<E>> operator()(const Label<1, Q> &j,
                                                                     const E &e) const {
    return {j.p, sym::Lit<bool>{{}, true}, sym::make_expr(e), true, radius, LNorm};
  }
};

/* eval(sum(i, [cond,] x)) (src/Symbolic.h): the sum over the row particles,
 * in storage order, of x -- a sum over j or an expression of i. */
template <typename P, typename T, typename C, typename X>
T eval(const sym::SumAll<P, T, C, X> &s) {
  constexpr unsigned BR = detail::BlockRows<T>::value;
  const size_t n = s.rows->size();
  std::vector<double> vals(n * BR, 0.0);
  const sym::HostRef<P> h(*s.rows);
  typename P::const_reference a = h.ref;
  const Vector<double, P::dimension> zero;
  if constexpr (sym::is_sum<X>::value) {
    vals = sym::sum_values(*s.rows, s.x);
  } else {
    const auto x = sym::make_expr(s.x);
    for (size_t i = 0; i < n; ++i) {
      a.index = int64_t(i);
      const T v = T(x.eval(zero, a, a));
      for (unsigned k = 0; k < BR; ++k) vals[i * BR + k] = detail::BlockRows<T>::get(v, k);
    }
  }
  T total = T();
  for (size_t i = 0; i < n; ++i) {
    a.index = int64_t(i);
    if (!s.c.eval(zero, a, a)) continue;
    if constexpr (BR == 1) {
      total = total + vals[i];
    } else {
      for (unsigned k = 0; k < BR; ++k) total[k] = total[k] + vals[i * BR + k];
    }
  }
  return total;
}

/* s[i] as the target of an assignment, s[i] / s[j] inside an expression */
template <typename Tag, int L, typename P> struct SymbolAt : sym::VarAt<Tag, L> {
  const P *p;

  template <typename Q, typename T, typename C, typename E>
  void operator=(const sym::Sum<Q, T, C, E> &s) const {
    assign(s, false);
  }
  template <typename Q, typename T, typename C, typename E>
  void operator+=(const sym::Sum<Q, T, C, E> &s) const {
    assign(s, true);
  }
  /* s[i] = expr of the row label only (univariate), evaluated on the host */
  template <typename E, typename = typename std::enable_if<!std::is_same<
                            typename std::decay<E>::type, SymbolAt>::value>::type>
  void operator=(const E &e) const {
    univariate(sym::make_expr(e));
  }
  void operator=(const SymbolAt &o) const { univariate(o); }

 private:
  template <typename X> void univariate(const X &x) const {
    static_assert(L == 0, "assign to the row label (label 0)");
    P &pp = const_cast<P &>(*p);
    const size_t n = pp.size();
    typedef typename std::decay<decltype(detail::getter<Tag>::get(pp)[0])>::type V;
    std::vector<V> out(n);
    {
      const sym::HostRef<P> h(pp);
      typename P::const_reference a = h.ref;
      const Vector<double, P::dimension> zero;
      for (size_t i = 0; i < n; ++i) {
        a.index = int64_t(i);
        out[i] = V(x.eval(zero, a, a));
      }
    }
    auto &col = detail::getter<Tag>::get(pp);
    for (size_t i = 0; i < n; ++i) col[i] = out[i];
    if (detail::is_position<Tag>::value && pp.searched()) pp.update_positions();
  }

  template <typename Q, typename T, typename C, typename E>
  void assign(const sym::Sum<Q, T, C, E> &s, bool add) const {
    static_assert(L == 0, "assign to the row label (label 0)");
    const size_t n = p->size();
    constexpr unsigned BR = detail::BlockRows<T>::value;
    const std::vector<double> c = sym::sum_values(*p, s);
    auto &col = detail::getter<Tag>::get(const_cast<P &>(*p));
    typedef typename std::decay<decltype(col[0])>::type V;
    for (size_t i = 0; i < n; ++i) {
      V v = add ? col[i] : V();
      if constexpr (BR == 1) {
        v = V(double(v) + c[i]);
      } else {
        for (unsigned k = 0; k < BR; ++k) v[k] = v[k] + c[i * BR + k];
      }
      col[i] = v;
    }
    if (detail::is_position<Tag>::value && p->searched()) const_cast<P &>(*p).update_positions();
  }
};

/* Symbol<Tag> (src/Symbolic.h): a variable, indexed by a label. */
template <typename Tag> struct Symbol {
  template <int L, typename P> SymbolAt<Tag, L, P> operator[](const Label<L, P> &l) const {
    SymbolAt<Tag, L, P> s;
    s.p = l.p;
    return s;
  }
};

}  // namespace Aboria

#endif  // ABORIA_GB_SYMBOLIC_CUH_
