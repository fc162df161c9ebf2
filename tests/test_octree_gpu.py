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


@pytest.mark.parametrize("dim,periodic,lnorm", [(3, False, 2), (2, True, 2), (3, True, -1),
                                                (2, False, 1)])
def test_radius_queries_on_the_octree(dim, periodic, lnorm):
    """The reference's HyperOctree answers the same radius queries as its cell
    lists (tree_query_iterator, src/NeighbourSearchBase.h:1438-1718).  On an
    octree particle set the GPU search gives the oracle's neighbour counts
    and sets, bit-exact, for stored and foreign query points; columns are
    storage indices of the octree order."""
    pos = workloads.uniform(20000, dim, seed=60 + dim)
    lo, hi, per = [0.0] * dim, [1.0] * dim, [periodic] * dim
    p = ab.Particles(dim).set(pos)
    p.init_octree(lo, hi, per, 32)
    cl = oracle.celllist_build(p.positions, lo, hi, per)
    q = np.concatenate([p.positions[:2000],
                        workloads.uniform(500, dim, lo=-0.1, hi=1.1, seed=70 + dim)])
    r = 0.05 if dim == 3 else 0.02
    counts = ab.radius_count(p, q, r, lnorm=lnorm)
    assert np.array_equal(counts, oracle.radius_count(cl, q, r, lnorm))
    rowptr, cols = ab.radius_query_csr(p, q, r, lnorm=lnorm)
    orp, ocols, _ = oracle.radius_lists(cl, q, r, lnorm=lnorm)
    assert np.array_equal(rowptr, orp)
    for i in range(len(q)):
        a = np.sort(cols[rowptr[i]:rowptr[i + 1]])
        b = np.sort(cl.perm[ocols[orp[i]:orp[i + 1]]])
        assert np.array_equal(a, b), i
