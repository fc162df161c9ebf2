// The reference's Level-3 symbolic expressions (src/Symbolic.h) through
// aboria_gb/symbolic.cuh, built by nvcc.
//
//   symbolic_test kat             the known answers of the reference's
//                                 tests/symbolic.h helper_neighbours (two
//                                 particles in a periodic [-1,1]^3): prints
//                                 "kat ok" or the first mismatch
//   symbolic_test run IN OUT      random particles from IN (n, r, then n x 3
//                                 positions), writes OUT/{ids,count,spring,
//                                 dense}.bin for the Python test's brute force
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "aboria_gb/Aboria.h"

using namespace Aboria;

ABORIA_VARIABLE(scalar, double, "scalar")
ABORIA_VARIABLE(count, int, "number of surrounding particles")
ABORIA_VARIABLE(spring, vdouble3, "linear spring force")
ABORIA_VARIABLE(dense_sum, double, "sum over every particle")

static int fail(const char *what, double got, double want) {
  std::printf("kat mismatch: %s: %.17g != %.17g\n", what, got, want);
  return 1;
}

// tests/symbolic.h helper_neighbours
static int kat() {
  typedef Particles<std::tuple<scalar>, 3> P;
  typedef position_d<3> position;
  P particles;
  const vdouble3 min(-1, -1, -1), max(1, 1, 1);
  const vbool3 periodic(true, true, true);
  const double diameter = 0.1;
  particles.init_neighbour_search(min, max, periodic);
  Symbol<position> p;
  Symbol<id> id_;
  Symbol<scalar> s;
  Label<0, P> a(particles);
  Label<1, P> b(particles);
  AccumulateWithinDistance<std::plus<double>> sum(diameter);
  particles.push_back(vdouble3(0, 0, 0));
  particles.push_back(vdouble3(diameter * 2, 0, 0));

  s[a] = sum(b, 1);
  if (get<scalar>(particles)[0] != 1) return fail("s[0] = sum(b, 1)", get<scalar>(particles)[0], 1);
  if (get<scalar>(particles)[1] != 1) return fail("s[1] = sum(b, 1)", get<scalar>(particles)[1], 1);

  p[a] = if_else(id_[a] == 0, vdouble3(diameter / 2.0, 0, 0), vdouble3(0, 0, 0));
  const double want0[2][3] = {{diameter / 2.0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < 2; ++i)
    for (int d = 0; d < 3; ++d)
      if (get<position>(particles)[i][d] != want0[i][d])
        return fail("p[a] = if_else(...)", get<position>(particles)[i][d], want0[i][d]);

  p[a] = 0.5 * (p[a] + s[a]);
  const double want1[2][3] = {{0.5 * (diameter / 2.0 + 1), 0.5, 0.5}, {0.5, 0.5, 0.5}};
  for (int i = 0; i < 2; ++i)
    for (int d = 0; d < 3; ++d)
      if (get<position>(particles)[i][d] != want1[i][d])
        return fail("p[a] = 0.5 * (p[a] + s[a])", get<position>(particles)[i][d], want1[i][d]);

  s[a] = sum(b, 1);
  if (get<scalar>(particles)[0] != 2) return fail("s[0] = sum(b, 1) again", get<scalar>(particles)[0], 2);
  if (get<scalar>(particles)[1] != 2) return fail("s[1] = sum(b, 1) again", get<scalar>(particles)[1], 2);

  Accumulate<std::plus<double>> sum_all;
  const double sum_of_sum = eval(sum_all(a, sum(b, 1.0)));
  if (sum_of_sum != 4) return fail("eval(sum_all(a, sum(b, 1.0)))", sum_of_sum, 4);

  p[a] = if_else(id_[a] == 0, vdouble3(0, 0, 0),
                 vdouble3(diameter / 2.0, diameter / 2.0, diameter / 2.0));
  s[a] = if_else(id_[a] == 0, 0, 1);
  if (get<scalar>(particles)[0] != 0) return fail("s = if_else(...)[0]", get<scalar>(particles)[0], 0);
  if (get<scalar>(particles)[1] != 1) return fail("s = if_else(...)[1]", get<scalar>(particles)[1], 1);

  AccumulateWithinDistance<std::plus<vdouble3>> sumVect(diameter);
  Accumulate<std::plus<vdouble3>> sum_all_vect;
  const vdouble3 sum_of_sumv =
      eval(sum_all_vect(a, sumVect(b, vdouble3(0, 0, 0) + 0.5 * (s[a] / 2.0 + s[b] / 10.0))));
  for (int d = 0; d < 3; ++d)
    if (std::fabs(sum_of_sumv[d] - 0.6) > 10 * 2.220446049250313e-16)
      return fail("eval(sum_all_vect(...))", sum_of_sumv[d], 0.6);
  p[a] = sumVect(b, vdouble3(0, 0, 0) + 0.5 * (s[a] / 2.0 + s[b] / 10.0));
  const double want2[2] = {0.05, 0.55};
  for (int i = 0; i < 2; ++i)
    for (int d = 0; d < 3; ++d)
      if (get<position>(particles)[i][d] != want2[i])
        return fail("p[a] = sumVect(b, ...)", get<position>(particles)[i][d], want2[i]);

  // the inf-norm range sum
  AccumulateWithinDistance<std::plus<double>, -1> box_sum(diameter);
  get<position>(particles)[0] = vdouble3(0, 0, 0);
  get<position>(particles)[1] = vdouble3(0.99 * diameter, 0.99 * diameter, 0.99 * diameter);
  particles.update_positions();
  s[a] = sum(b, 1);
  if (get<scalar>(particles)[0] != 1) return fail("s = sum(b, 1), 2-norm", get<scalar>(particles)[0], 1);
  if (get<scalar>(particles)[1] != 1) return fail("s = sum(b, 1), 2-norm", get<scalar>(particles)[1], 1);
  s[a] = box_sum(b, 1);
  if (get<scalar>(particles)[0] != 2) return fail("s = box_sum(b, 1)", get<scalar>(particles)[0], 2);
  if (get<scalar>(particles)[1] != 2) return fail("s = box_sum(b, 1)", get<scalar>(particles)[1], 2);

  // tests/neighbours.h helper_single_particle: searches with a scale transform
  {
    typedef Particles<std::tuple<scalar>, 3> T1;
    T1 test;
    test.init_neighbour_search(vdouble3(-1, -1, -1), vdouble3(1, 1, 1), vbool3(true, true, true));
    const double radius = 0.1;
    test.push_back(vdouble3(0, 0, 0));
    if (euclidean_search(test, vdouble3(radius / 2, radius / 2, 0), radius).size() != 1)
      return fail("euclidean_search count", 0, 1);
    if (euclidean_search(test, vdouble3(2 * radius, 0, 0), radius).size() != 0)
      return fail("euclidean_search count far", 1, 0);
    const auto scale = create_scale_transform(vdouble3(1.0 / radius, 1.0 / radius, 1.0 / radius));
    if (euclidean_search(test, vdouble3(radius / 2, radius / 2, 0), 1.0, scale).size() != 1)
      return fail("scaled euclidean_search count", 0, 1);
    if (euclidean_search(test, vdouble3(2 * radius, 0, 0), 1.0, scale).size() != 0)
      return fail("scaled euclidean_search count far", 1, 0);
    struct Skew {
      vdouble3 operator()(const vdouble3 &v) const { return vdouble3(v[0] + 0.3 * v[1], v[1], v[2]); }
    };
    const auto skew = create_linear_transform<3>(Skew());
    // (0.05, 0.2, 0) from the particle: |skew dx| = |(0.11, 0.2, 0)| < 0.25 < |dx| * 1.2
    const auto hits = euclidean_search(test, vdouble3(-0.05, -0.2, 0), 0.25, skew);
    if (hits.size() != 1) return fail("skewed euclidean_search count", double(hits.size()), 1);
    if (hits[0].dx[0] != 0.05 + 0.3 * 0.2) return fail("skewed dx", hits[0].dx[0], 0.05 + 0.3 * 0.2);
  }
  std::printf("kat ok\n");
  return 0;
}

template <typename T> static void write(const std::string &path, const std::vector<T> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), std::streamsize(v.size() * sizeof(T)));
}

// random particles in the unit cube: the count and the linear spring sum of
// tests/speed_test.h:756-836 (self pair excluded with if_else), and a dense
// sum over every particle
static int run(const char *in, const char *out) {
  std::ifstream f(in, std::ios::binary);
  int64_t n = 0;
  double r = 0;
  f.read(reinterpret_cast<char *>(&n), 8);
  f.read(reinterpret_cast<char *>(&r), 8);
  std::vector<double> xyz(size_t(n) * 3);
  f.read(reinterpret_cast<char *>(xyz.data()), std::streamsize(xyz.size() * 8));
  typedef Particles<std::tuple<count, spring, dense_sum>, 3> P;
  P nodes;
  for (int64_t i = 0; i < n; ++i) nodes.push_back(vdouble3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
  nodes.init_neighbour_search(vdouble3(0, 0, 0), vdouble3(1, 1, 1), vbool3(false, false, false));
  Symbol<count> c;
  Symbol<spring> a;
  Symbol<dense_sum> ds;
  Label<0, P> i(nodes);
  Label<1, P> j(nodes);
  auto dx = create_dx(i, j);
  Accumulate<std::plus<int>> sumi;
  Accumulate<std::plus<vdouble3>> sum;
  Accumulate<std::plus<double>> sumd;
  c[i] = sumi(j, norm(dx) < r, 1);
  a[i] = sum(j, norm(dx) < r,
             if_else(norm(dx) > 0, (r - norm(dx)) / norm(dx) * dx, vdouble3(0, 0, 0)));
  ds[i] = sumd(j, true, 1.0 / (1.0 + norm(dx) * norm(dx)));
  const std::string o(out);
  write(o + "/ids.bin", get<id>(nodes));
  std::vector<double> pos;
  for (const auto &x : get<position_d<3>>(static_cast<const P &>(nodes)))
    for (unsigned d = 0; d < 3; ++d) pos.push_back(x[d]);
  write(o + "/pos.bin", pos);
  write(o + "/count.bin", get<count>(nodes));
  std::vector<double> sp;
  for (const auto &v : get<spring>(nodes))
    for (unsigned d = 0; d < 3; ++d) sp.push_back(v[d]);
  write(o + "/spring.bin", sp);
  write(o + "/dense.bin", get<dense_sum>(nodes));
  return 0;
}

int main(int argc, char **argv) {
  if (argc >= 2 && std::strcmp(argv[1], "kat") == 0) return kat();
  if (argc >= 4 && std::strcmp(argv[1], "run") == 0) return run(argv[2], argv[3]);
  std::fprintf(stderr, "usage: symbolic_test kat | run IN OUT\n");
  return 2;
}
