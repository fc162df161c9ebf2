"""GPU HyperOctree vs the oracle: tag order and leaves bit-exact."""
import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,n,n_leaf", [(3, 100000, 64), (2, 200000, 256), (3, 5000, 10),
                                          (2, 1000, 1), (1, 3000, 16)])
def test_octree_matches_oracle(dim, n, n_leaf):
    pos = workloads.uniform(n, dim, seed=50 + dim)
    if dim == 3 and n == 5000:
        pos = workloads.gaussian_mixture(n, 3, seed=51)
    p = ab.Particles(dim).set(pos)
    p.init_octree([0.0] * dim, [1.0] * dim, [False] * dim, n_leaf)
    t = oracle.octree_build(pos, [0.0] * dim, [1.0] * dim, n_leaf)
    assert np.array_equal(p.ids, t.perm)
    assert np.array_equal(p.positions, pos[t.perm])
    lv, lt, lb, le = p.tree_leaves()
    assert np.array_equal(lv, t.leaf_level) and np.array_equal(lt, t.leaf_tag)
    assert np.array_equal(lb, t.leaf_begin) and np.array_equal(le, t.leaf_end)
    assert np.all(le - lb <= n_leaf) or np.any(lv == 32 // dim - 2)


def test_octree_sparse_operator_works():
    pos = workloads.uniform(20000, 2, seed=52)
    p = ab.Particles(2).set(pos)
    p.init_octree([0, 0], [1, 1], [False, False], 32)
    cl = oracle.celllist_build(p.positions, [0, 0], [1, 1], [False, False])
    b = np.random.default_rng(53).standard_normal(len(p))
    K = ab.create_sparse_operator(p, p, 0.05, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, 400.0))
    # oracle rows in octree storage order; columns through the oracle's cell order
    ref = oracle.sparse_matvec(cl, p.positions, 0.05, ab.K_COMPACT_GAUSSIAN, [400.0], b[cl.perm])
    c = K * b
    assert np.linalg.norm(c - ref) / np.linalg.norm(ref) < 1e-12
