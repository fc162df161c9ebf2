"""Full-size checks on the sparse-operator workload (N = 4,194,304: 16-Gaussian
mixture + 20% uniform, periodic unit box, r = 0.02), where the oracle is too
slow to run: size-independent properties of the cell list, the radius search
and the operator.

* Sortedness and bucket ranges of the cell list; rebuilding is idempotent.
* A checksum of checksums: K * 1 with the constant kernel (value 1) is, row
  by row, the neighbour count -- in FP64 and in mixed precision (FP32 blocks of
  ones are exact) it must equal the radius-count kernel's counts exactly, so
  the matvec's neighbour sets agree with the search's at full size.
* Linearity of the mixed Wendland operator; symmetry of the FP64 one
  (b1 . K b2 = b2 . K b1, the kernel being symmetric and rows == cols).
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import workloads

pytestmark = pytest.mark.gpu

N, R = 4_194_304, 0.02


@pytest.fixture(scope="module")
def cfg2():
    pos = workloads.gaussian_mixture(N, 3, k=16, sigma=0.03, frac_uniform=0.2, seed=2024,
                                     periodic=True)
    p = ab.Particles(3).set(pos)
    p.init_neighbour_search([0, 0, 0], [1, 1, 1], [True] * 3, 10.0)
    return p


def test_cell_list_sorted_and_idempotent(cfg2):
    p = cfg2
    bb, be, keys = p.buckets()
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    assert np.all(be >= bb) and int((be - bb).astype(np.int64).sum()) == N
    nz = be > bb
    assert np.all(keys[bb[nz]] == np.nonzero(nz)[0])
    ids = p.ids
    p.init_neighbour_search([0, 0, 0], [1, 1, 1], [True] * 3, 10.0)
    assert np.array_equal(p.ids, ids)


def test_constant_kernel_matvec_equals_counts(cfg2):
    p = cfg2
    counts = ab.radius_count(p, p.positions, R).astype(np.float64)
    assert counts.min() >= 1  # every particle is its own neighbour
    ones = np.ones(N)
    kern = ab.Kernel.make(ab.K_CONST, 1.0)
    for prec in (ab.PREC_MIXED, ab.PREC_FP64):
        K = ab.create_sparse_operator(p, p, R, kern, prec)
        c = K * ones
        assert np.array_equal(c, counts), prec
        del K


def test_linearity_and_symmetry(cfg2):
    p = cfg2
    rng = np.random.default_rng(7)
    b1, b2 = rng.standard_normal(N), rng.standard_normal(N)
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1.0 / R)
    K32 = ab.create_sparse_operator(p, p, R, kern, ab.PREC_MIXED)
    k1, k2 = K32 * b1, K32 * b2
    k12 = K32 * (2.0 * b1 + b2)
    assert np.linalg.norm(k12 - (2.0 * k1 + k2)) / np.linalg.norm(k12) < 2e-6
    del K32
    K64 = ab.create_sparse_operator(p, p, R, kern, ab.PREC_FP64)
    a, b = b1 @ (K64 * b2), b2 @ (K64 * b1)
    assert abs(a - b) <= 1e-10 * (abs(a) + abs(b))
