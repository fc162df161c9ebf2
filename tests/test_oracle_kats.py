"""Pins the CPU oracle against the reference's own known-answer tests.

Every expected value comes from tests/golden/reference_kats.json, which
transcribes the reference test files (cited per entry).  No GPU needed.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
import workloads

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.mark.parametrize("case", KATS["bucket_collapse"])
def test_bucket_collapse_reassemble(case):
    assert oracle.collapse(case["size"], case["index_vector"]) == case["index"]
    assert list(oracle.reassemble(case["size"], case["index"])) == case["index_vector"]


@pytest.mark.parametrize("case", KATS["point_to_bucket"])
def test_point_to_bucket(case):
    size = np.array(case["size"])
    side = (np.array(case["hi"], float) - np.array(case["lo"], float)) / size
    idx, v = oracle.point_to_bucket(size, case["lo"], side, case["point"])
    assert list(v) == case["bucket_vector"]
    assert idx == case["index"]


def test_sparse_operator_kat():
    k = KATS["sparse_operator"]
    pos = np.array(k["positions"])
    cl = oracle.celllist_build(pos, k["domain_lo"], k["domain_hi"], k["periodic"])
    # storage order after the cell sort; map the answer through ids
    ids = cl.perm
    s1 = np.full(3, k["scalar1"])
    s2 = np.full(3, k["scalar2"])
    v = np.array(k["v"], float)[ids]
    c = oracle.sparse_matvec(cl, cl.pos, k["radius"], 6, [], v, row_s=s1, col_s=s2)
    ans = np.empty(3)
    ans[ids] = c
    assert list(ans) == k["answer"]
    rowptr, cols, _ = oracle.radius_lists(cl, cl.pos, k["radius"])
    assert rowptr[-1] == k["nonzeros"]


def test_dense_operator_kat():
    k = KATS["dense_operator"]
    pos = np.array(k["positions"])
    for case in k["cases"]:
        c = oracle.dense_matvec(pos, pos, 6, [], np.array(case["v"], float),
                                row_s=np.full(3, k["scalar1"]), col_s=np.full(3, k["scalar2"]))
        assert list(c) == case["answer"]


def gauss_circle(r):
    n = 0
    for i in range(100):
        n += int(math.floor(r ** 2 / (4 * i + 1))) - int(math.floor(r ** 2 / (4 * i + 3)))
    return 1 + 4 * n


@pytest.mark.parametrize("case", KATS["regular_lattice_l2"]["cases"])
def test_regular_lattice_counts(case):
    d, n = case["dim"], case["n"]
    pos = workloads.lattice(n, d)
    cl = oracle.celllist_build(pos, [0.0] * d, [float(n)] * d, [True] * d, case["n_leaf"])
    counts = oracle.radius_count(cl, cl.pos, case["r"])
    assert np.all(counts == gauss_circle(case["r"]))


@pytest.mark.parametrize("case", KATS["regular_lattice_linf"]["cases"])
def test_regular_lattice_box_counts(case):
    """The reference's box search (chebyshev norm) on the periodic lattice:
    (2 floor(r) + 1)^D neighbours for every point."""
    d, n = case["dim"], case["n"]
    pos = workloads.lattice(n, d)
    cl = oracle.celllist_build(pos, [0.0] * d, [float(n)] * d, [True] * d, case["n_leaf"])
    counts = oracle.radius_count(cl, cl.pos, case["r"], lnorm=-1)
    assert np.all(counts == (2 * int(np.floor(case["r"])) + 1) ** d)


def _brute_norm_counts(pos, L, periodic, r, lnorm):
    """Independent numpy restatement: minimum-image offsets (exact while r <
    L/2), then sum dx^2 <= r^2, sum |dx| <= r or max |dx| <= r."""
    out = np.zeros(len(pos), np.int64)
    for s in range(0, len(pos), 256):
        dx = pos[None, :, :] - pos[s:s + 256, None, :]
        if periodic:
            dx -= L * np.round(dx / L)
        a = np.abs(dx)
        if lnorm == 2:
            ok = (dx * dx).sum(-1) <= r * r
        elif lnorm == 1:
            ok = a.sum(-1) <= r
        else:
            ok = a.max(-1) <= r
        out[s:s + 256] = ok.sum(1)
    return out


@pytest.mark.parametrize("lnorm", [2, 1, -1])
@pytest.mark.parametrize("periodic", [False, True])
def test_norm_searches_vs_brute_force(lnorm, periodic):
    """manhatten_search / chebyshev_search / euclidean_search counts
    (src/Search.h:797-845) against a brute force, 3-D, r below half the box."""
    pos = workloads.uniform(3000, 3, seed=4100)
    cl = oracle.celllist_build(pos, [0.0] * 3, [1.0] * 3, [periodic] * 3, 10.0)
    r = 0.12
    counts = oracle.radius_count(cl, cl.pos, r, lnorm=lnorm)
    assert np.array_equal(counts, _brute_norm_counts(cl.pos, 1.0, periodic, r, lnorm))


@pytest.mark.parametrize("case", KATS["random_brute_force"]["cases"])
def test_random_counts_vs_brute_force(case):
    d = case["dim"]
    pos = workloads.float_uniform(case["N"], d, seed=1234 + d)
    lo, hi = [-1.0] * d, [1.0] * d
    cl = oracle.celllist_build(pos, lo, hi, [case["periodic"]] * d, case["n_leaf"])
    counts = oracle.radius_count(cl, cl.pos, case["r"])
    brute = oracle.brute_counts(cl.pos, lo, hi, case["periodic"], case["r"])
    assert np.array_equal(counts, brute)


def test_stable_and_stl_orders_agree_on_cells():
    pos = workloads.uniform(5000, 3, seed=3)
    a = oracle.celllist_build(pos, [0] * 3, [1] * 3, [False] * 3, stable=True)
    b = oracle.celllist_build(pos, [0] * 3, [1] * 3, [False] * 3, stable=False)
    assert np.array_equal(a.keys, b.keys)
    assert np.array_equal(a.begin, b.begin) and np.array_equal(a.end, b.end)
    for c in np.flatnonzero(a.end > a.begin)[:500]:
        s = slice(a.begin[c], a.end[c])
        assert set(a.perm[s]) == set(b.perm[s])
    # stable order: original index ascending within a bucket
    for c in np.flatnonzero(a.end - a.begin > 1)[:500]:
        s = slice(a.begin[c], a.end[c])
        assert np.all(np.diff(a.perm[s]) > 0)


def test_grid_matches_reference_formula():
    # cfg1: N=1e5, unit cube, n_leaf=10 -> 21^3 buckets of side 1/21
    size, side, nc = oracle.grid(3, [0] * 3, [1] * 3, [False] * 3, 10.0, 100000)
    assert list(size) == [21, 21, 21] and nc == 9261
    # cfg2: N=4,194,304 -> 74^3
    size, side, nc = oracle.grid(3, [0] * 3, [1] * 3, [True] * 3, 10.0, 4194304)
    assert list(size) == [74, 74, 74] and nc == 405224


def test_grid_hysteresis_rule():
    """The grid is kept while the alive count stays within [0.5, 2] x the count
    it was computed with (src/CellListOrdered.h:133-136)."""
    pos = workloads.uniform(1000, 3, seed=61)
    fresh = oracle.celllist_build(pos, [0] * 3, [1] * 3, [False] * 3, 10.0)
    assert list(fresh.size) == [4, 4, 4]
    kept = oracle.celllist_build(pos, [0] * 3, [1] * 3, [False] * 3, 10.0, prev_grid_n=1900)
    assert list(kept.size) == list(oracle.grid(3, [0] * 3, [1] * 3, [False] * 3, 10.0, 1900)[0])
    assert list(kept.size) != list(fresh.size)
    again = oracle.celllist_build(pos, [0] * 3, [1] * 3, [False] * 3, 10.0, prev_grid_n=2100)
    assert list(again.size) == list(fresh.size)  # 1000 < 0.5 x 2100: recomputed


def test_periodic_wrap_and_deletion():
    pos = np.array([[1.25, 0.5], [-0.25, 0.5], [0.5, 0.5], [0.5, np.nan]])
    cl = oracle.celllist_build(pos, [0, 0], [1, 1], [True, True], 1.0)
    assert cl.n == 3  # the NaN particle is deleted
    got = sorted(map(tuple, cl.pos))
    assert got == sorted([(0.25, 0.5), (0.75, 0.5), (0.5, 0.5)])
    cl = oracle.celllist_build(pos, [0, 0], [1, 1], [False, False], 1.0)
    assert cl.n == 1  # outside a non-periodic domain -> deleted


def test_octree_leaves_partition_and_sizes():
    pos = workloads.uniform(20000, 3, seed=60)
    t = oracle.octree_build(pos, [0] * 3, [1] * 3, 64)
    assert np.all(np.diff(t.tags) >= 0)
    order = np.argsort(t.leaf_begin)
    b, e = t.leaf_begin[order], t.leaf_end[order]
    assert b[0] == 0 and e[-1] == 20000 and np.array_equal(b[1:], e[:-1])
    assert np.all(e - b <= 64)
    # a leaf's particles all carry its tag prefix
    for i in range(0, len(t.leaf_tag), 37):
        shift = (8 - t.leaf_level[i]) * 3
        assert np.all((t.tags[t.leaf_begin[i]:t.leaf_end[i]] >> shift) == (t.leaf_tag[i] >> shift))


def test_mlp_oracle_gradient_matches_finite_differences():
    import mlp_oracle
    rng = np.random.default_rng(90)
    dims = [6, 5, 5, 3]
    n = sum(dims[i] * dims[i + 1] + dims[i + 1] for i in range(3))
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((7, 6))
    y = rng.standard_normal((7, 3))
    sc, sh = np.array([2.0, 1.0, 0.5]), np.array([0.1, -0.2, 0.0])
    loss, g = mlp_oracle.loss_and_grad(p, dims, x, y, sc, sh)
    for i in rng.choice(n, 12, replace=False):
        e = np.zeros(n)
        e[i] = 1e-6
        lp, _ = mlp_oracle.loss_and_grad(p + e, dims, x, y, sc, sh)
        lm, _ = mlp_oracle.loss_and_grad(p - e, dims, x, y, sc, sh)
        assert abs((lp - lm) / 2e-6 - g[i]) < 1e-6 * max(1.0, abs(g[i]))


def test_mlp_oracle_residual_gradient_matches_finite_differences():
    """The approximate-inverse residual loss: k = 4 support points in 2-D."""
    import mlp_oracle
    rng = np.random.default_rng(95)
    dims = [8, 6, 4]
    n = sum(dims[i] * dims[i + 1] + dims[i + 1] for i in range(2))
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((5, 8))
    x[:, :2] = 0.0  # f_0 is the row's own point
    sc, sh = np.full(4, 0.3), np.array([1.0, 0.0, 0.0, 0.0])
    kern = lambda d2: np.exp(-d2)
    loss, g = mlp_oracle.residual_loss_and_grad(p, dims, x, 2, kern, 2.5, sc, sh)
    for i in rng.choice(n, 12, replace=False):
        e = np.zeros(n)
        e[i] = 1e-6
        lp, _ = mlp_oracle.residual_loss_and_grad(p + e, dims, x, 2, kern, 2.5, sc, sh)
        lm, _ = mlp_oracle.residual_loss_and_grad(p - e, dims, x, 2, kern, 2.5, sc, sh)
        assert abs((lp - lm) / 2e-6 - g[i]) < 1e-6 * max(1.0, abs(g[i]))


@pytest.mark.parametrize("dim", [2, 3])
def test_fmm_oracle_reference_kat(dim):
    """tests/fmm.h:167-253: N=1000 uniform, n_leaf 10, kernel sqrt(|dx|^2 + 0.01),
    source prod cos(2 pi x)/N; order 3 must give L2^2/scale < 1e-2."""
    N = 1000
    pos = workloads.uniform(N, dim, seed=110 + dim)
    b = np.prod(np.cos(2 * np.pi * pos), axis=1) / N
    direct = oracle.direct_sum(pos, 5, [0.01], b, np.arange(N))
    scale = np.sum(direct ** 2)
    for order in (3, 5):
        c = oracle.fmm(pos, [0.0] * dim, [1.0] * dim, 10, order, 5, [0.01], b)
        l2 = np.sum((c - direct) ** 2)
        if order == 3:
            assert l2 / scale < 1e-2
    assert l2 / scale < 1e-6  # order 5 is far more accurate on this smooth kernel
