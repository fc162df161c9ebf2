// Drives the C++ mirror of Aboria's API (include/aboria_gb/Aboria.h) the way
// the reference's own tests use Aboria (tests/neighbours.h, tests/operators.h,
// tests/rbf_interpolation.h, tests/fmm.h), and writes what it computed to
// binary files that tests/test_cpp_api.py compares with the oracle.
//
// Compiles as C++ (g++ -x c++) or CUDA (nvcc; adds the user-functor operator).
//   api_test trap            -> a failing call prints and raises SIGTRAP
//   api_test throw           -> (built with -DABORIA_GB_THROW) the failure is
//                               a std::runtime_error; prints "caught: ..."
//   api_test run IN OUTDIR   -> the parity workload
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "aboria_gb/Aboria.h"

using namespace Aboria;

typedef Particles<std::tuple<>, 3> Cells3;
typedef Particles<std::tuple<>, 3, void, HyperOctree> Tree3;

template <typename T> static void write(const std::string &path, const std::vector<T> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), std::streamsize(v.size() * sizeof(T)));
}

#ifdef __CUDACC__
ABORIA_VARIABLE(scalar1, double, "scalar1")
ABORIA_VARIABLE(scalar2, double, "scalar2")
ABORIA_VARIABLE(search_radius, double, "search_radius")
typedef Particles<std::tuple<scalar1, scalar2>> ParticlesType;  // D = 3, as the reference's default
typedef Particles<std::tuple<search_radius>, 3> RadiusParticles;
#endif

static int run(const char *in, const std::string &out) {
  std::ifstream f(in, std::ios::binary);
  int64_t hdr[2];
  f.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
  const int64_t n = hdr[0], nq = hdr[1];
  double prm[2];  // radius, Wendland radius of the solve
  f.read(reinterpret_cast<char *>(prm), sizeof(prm));
  std::vector<double> pos(static_cast<size_t>(n) * 3), b(static_cast<size_t>(n)),
      q(static_cast<size_t>(nq) * 3);
  f.read(reinterpret_cast<char *>(pos.data()), std::streamsize(pos.size() * 8));
  f.read(reinterpret_cast<char *>(b.data()), std::streamsize(b.size() * 8));
  f.read(reinterpret_cast<char *>(q.data()), std::streamsize(q.size() * 8));
  if (!f) {
    std::fprintf(stderr, "short input file\n");
    return 2;
  }
  const double r = prm[0];

  // tests/neighbours.h pattern: push_back, init_neighbour_search, euclidean_search
  Cells3 particles;
  for (int64_t i = 0; i < n; ++i)
    particles.push_back(vdouble3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
  particles.init_neighbour_search(vdouble3(0, 0, 0), vdouble3(1, 1, 1), vbool3(false, false, false));
  const std::vector<int64_t> &ids = get<id>(particles);
  write(out + "/ids.bin", ids);

  std::vector<int32_t> counts, lists;
  for (int64_t k = 0; k < nq; ++k) {
    const vdouble3 x(q[3 * k], q[3 * k + 1], q[3 * k + 2]);
    auto res = euclidean_search(particles, x, r);
    counts.push_back(int32_t(res.size()));
    for (auto &s : res) {
      // dx must be the separation of the stored particle from x
      const auto &pj = get<position>(particles)[size_t(s.index)];
      for (int d = 0; d < 3; ++d)
        if (s.dx[d] != pj[d] - x[d]) {
          std::fprintf(stderr, "dx mismatch\n");
          return 3;
        }
      lists.push_back(s.index);
    }
  }
  write(out + "/counts.bin", counts);
  write(out + "/lists.bin", lists);

  {
    // push_back / find-by-id / erase on the searchable set (src/Particles.h:
    // 264-389, src/NeighbourSearchBase.h:276-321); the copy keeps the set
    // used below unchanged
    Cells3 edit;
    for (int64_t i = 0; i < n; ++i)
      edit.push_back(vdouble3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    edit.init_neighbour_search(vdouble3(0, 0, 0), vdouble3(1, 1, 1), vbool3(false, false, false));
    edit.push_back(vdouble3(0.123, 0.456, 0.789));
    const int64_t new_id = n;  // ids run 0..n-1 for the first n particles
    const size_t at = edit.find(new_id);
    const auto &xp = get<position>(edit)[at];
    std::vector<double> res = {double(edit.size()), double(at < edit.size()),
                               xp[0], xp[1], xp[2]};
    edit.erase(at);
    res.push_back(double(edit.size()));
    res.push_back(double(edit.find(new_id) == edit.size()));
    res.push_back(double(edit.find(7) < edit.size() && get<id>(edit)[edit.find(7)] == 7));
    write(out + "/edit.bin", res);
  }

  // tests/operators.h pattern: K = create_sparse_operator(...); c = K * b
  std::vector<double> bs(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) bs[size_t(i)] = b[size_t(ids[size_t(i)])];
  const double c = r / 2;
  auto K = create_sparse_operator(particles, particles, r, kernels::gaussian(c));
  std::vector<double> kb = K * bs;
  write(out + "/kb.bin", kb);
#ifdef __CUDACC__
  {
    // the Gaussian as a user closure f(dx, a, b), matrix-free over the cell
    // list, against the built-in kernel: non-periodic and periodic
    const double inv_c2 = 1.0 / (c * c);
    auto gauss = [inv_c2] __host__ __device__(const vdouble3 &dx, Cells3::const_reference,
                                               Cells3::const_reference) {
      return exp(-dx.squaredNorm() * inv_c2);
    };
    auto Kf = create_sparse_operator(particles, particles, r, gauss);
    write(out + "/kf.bin", Kf * bs);
    Cells3 per;
    for (int64_t i = 0; i < n; ++i) per.push_back(vdouble3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    per.init_neighbour_search(vdouble3(0, 0, 0), vdouble3(1, 1, 1), vbool3(true, true, true));
    std::vector<double> bp(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) bp[size_t(i)] = b[size_t(get<id>(per)[size_t(i)])];
    auto Kp = create_sparse_operator(per, per, r, kernels::gaussian(c));
    auto Kfp = create_sparse_operator(per, per, r, gauss);
    write(out + "/kbp.bin", Kp * bp);
    write(out + "/kfp.bin", Kfp * bp);
  }
  {
    // tests/operators.h:810-963: three particles 0.09 apart, diameter 0.1,
    // scalar1 = 1 and scalar2 = 2 on every particle; the closure
    // get<scalar1>(a) + get<scalar2>(b) and the 2 x 1 block closure
    // (s1_a + s2_b, s1_a - s2_b)
    ParticlesType kat;
    const double diameter = 0.1;
    ParticlesType::value_type p;
    get<scalar1>(p) = 1.0;
    get<scalar2>(p) = 2.0;
    for (int q = 0; q < 3; ++q) {
      get<position>(p) = vdouble3(diameter * 0.9 * q, 0, 0);
      kat.push_back(p);
    }
    kat.init_neighbour_search(vdouble3(-1, -1, -1), vdouble3(1, 1, 1), vbool3(false, false, false));
    std::vector<double> v(3);
    for (int q = 0; q < 3; ++q) v[size_t(q)] = double(get<id>(kat)[size_t(q)] + 1);  // (1, 2, 3) by id
    auto C = create_sparse_operator(
        kat, kat, diameter,
        [] __host__ __device__(const vdouble3 &, ParticlesType::const_reference a,
                               ParticlesType::const_reference b) {
          return get<scalar1>(a) + get<scalar2>(b);
        });
    auto C2 = create_sparse_operator(
        kat, kat, diameter,
        [] __host__ __device__(const vdouble3 &, ParticlesType::const_reference a,
                               ParticlesType::const_reference b) {
          return Vector<double, 2>(get<scalar1>(a) + get<scalar2>(b),
                                   get<scalar1>(a) - get<scalar2>(b));
        });
    std::vector<double> a1 = C * v, a2 = C2 * v;
    std::vector<double> res;  // by id: answer, then block answer, then nnz
    std::vector<double> r1(3), r2(6);
    for (int q = 0; q < 3; ++q) {
      const int64_t pid = get<id>(kat)[size_t(q)];
      r1[size_t(pid)] = a1[size_t(q)];
      r2[size_t(2 * pid)] = a2[size_t(2 * q)];
      r2[size_t(2 * pid + 1)] = a2[size_t(2 * q + 1)];
    }
    res.insert(res.end(), r1.begin(), r1.end());
    res.insert(res.end(), r2.begin(), r2.end());
    res.push_back(double(C.nonzeros()));
    res.push_back(double(C2.nonzeros()));
    write(out + "/kat.bin", res);
  }
  {
    // tests/operators.h:969-1090: dense closures over particle variables, a
    // zero operator and the 2 x 2 block operator [A B; C 0]
    ParticlesType particles3, augment;
    const double diameter = 0.1;
    ParticlesType::value_type p;
    for (int q = 0; q < 3; ++q) {
      get<position>(p) = vdouble3(diameter * 0.9 * q, 0, 0);
      get<scalar1>(p) = q + 1;
      get<scalar2>(p) = 0.1 * (q + 1);
      particles3.push_back(p);
    }
    get<scalar1>(p) = 0;
    get<scalar2>(p) = 0;
    get<position>(p) = vdouble3(-diameter * 1.8, 0, 0);
    augment.push_back(p);
    particles3.init_neighbour_search(vdouble3(-1, -1, -1), vdouble3(1, 1, 1),
                                     vbool3(false, false, false));
    auto A = create_dense_operator(
        particles3, particles3,
        [] __host__ __device__(ParticlesType::const_reference a, ParticlesType::const_reference) {
          return get<scalar1>(a);
        });
    auto B = create_dense_operator(
        particles3, augment,
        [] __host__ __device__(ParticlesType::const_reference a, ParticlesType::const_reference) {
          return get<scalar2>(a);
        });
    auto Cd = create_dense_operator(
        augment, particles3,
        [] __host__ __device__(ParticlesType::const_reference, ParticlesType::const_reference b) {
          return get<scalar2>(b);
        });
    auto Zero = create_zero_operator(augment, augment);
    auto Full = create_block_operator<2, 2>(A, B, Cd, Zero);
    std::vector<double> ones(4, 1.0);
    std::vector<double> ans = Full * ones;
    ans.push_back(double(Full.rows()));
    ans.push_back(double(Full.cols()));
    write(out + "/block_kat.bin", ans);
  }
  {
    // create_sparse_operator(rows, cols, radius_function, f) with a per-row
    // search radius held in a particle variable
    RadiusParticles rp;
    RadiusParticles::value_type p;
    for (int64_t i = 0; i < n; ++i) {
      get<position>(p) = vdouble3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      get<search_radius>(p) = 0.02 + 0.06 * b[size_t(i)] * b[size_t(i)] / (1.0 + b[size_t(i)] * b[size_t(i)]);
      rp.push_back(p);
    }
    rp.init_neighbour_search(vdouble3(0, 0, 0), vdouble3(1, 1, 1), vbool3(false, false, false));
    const double inv_c2 = 1.0 / (c * c);
    auto Kv = create_sparse_operator(
        rp, rp,
        [] __host__ __device__(RadiusParticles::const_reference a) { return get<search_radius>(a); },
        [inv_c2] __host__ __device__(const vdouble3 &dx, RadiusParticles::const_reference,
                                     RadiusParticles::const_reference) {
          return exp(-dx.squaredNorm() * inv_c2);
        });
    std::vector<double> bv(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) bv[size_t(i)] = b[size_t(get<id>(rp)[size_t(i)])];
    write(out + "/kv.bin", Kv * bv);
    write(out + "/kv_radius.bin", get<search_radius>(rp));
    write(out + "/kv_ids.bin", get<id>(rp));
  }
#endif

  // tests/rbf_interpolation.h pattern: GMRES with SchwartzPreconditioner on an
  // octree particle set
  Tree3 tree;
  for (int64_t i = 0; i < n; ++i)
    tree.push_back(vdouble3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
  tree.init_neighbour_search(vdouble3(0, 0, 0), vdouble3(1, 1, 1), vbool3(false, false, false), 64);
  const double rw = prm[1];
  auto W = create_sparse_operator(tree, tree, rw, kernels::wendland_c2(rw));
  std::vector<double> rhs(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) rhs[size_t(i)] = b[size_t(get<id>(tree)[size_t(i)])];
  GMRES<Operator, SchwartzPreconditioner<>> gmres;
  gmres.set_restart(50);
  gmres.setMaxIterations(500);
  gmres.setTolerance(1e-10);
  gmres.compute(W);
  std::vector<double> x = gmres.solve(rhs);
  std::vector<double> wx = W * x;
  double rn = 0, bn = 0;
  for (int64_t i = 0; i < n; ++i) {
    rn += (rhs[size_t(i)] - wx[size_t(i)]) * (rhs[size_t(i)] - wx[size_t(i)]);
    bn += rhs[size_t(i)] * rhs[size_t(i)];
  }
  std::vector<double> solve = {double(gmres.iterations()), gmres.error(), std::sqrt(rn / bn)};
  write(out + "/solve.bin", solve);

  // tests/fmm.h pattern: create_fmm_operator<N>(particles, particles, kernel)
  auto F = create_fmm_operator<3>(tree, tree, kernels::multiquadric(0.01));
  std::vector<double> fb = F * rhs;
  write(out + "/fmm.bin", fb);
  write(out + "/tree_ids.bin", get<id>(tree));
  std::printf("ok n=%lld pairs-nonzero\n", (long long)n);
  return 0;
}

int main(int argc, char **argv) {
  const std::string mode = argc > 1 ? argv[1] : "";
  if (mode == "trap") {
    Cells3 p;              // no device: the context cannot be created
    p.update_positions();  // with a device: no search structure yet
    return 0;
  }
  if (mode == "throw") {
    try {
      Cells3 p;
      p.update_positions();
    } catch (const std::runtime_error &e) {
      std::printf("caught: %s\n", e.what());
      return 0;
    }
    return 1;
  }
  if (mode == "run" && argc == 4) return run(argv[2], argv[3]);
  std::fprintf(stderr, "usage: api_test trap|throw|run IN OUTDIR\n");
  return 2;
}
