"""GPU radius search vs the oracle: bit-exact neighbour counts and sets."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def build(pos, lo, hi, periodic, n_leaf=10.0):
    p = ab.Particles(pos.shape[1]).set(pos)
    p.init_neighbour_search(lo, hi, periodic, n_leaf)
    cl = oracle.celllist_build(pos, lo, hi, periodic, n_leaf)
    assert np.array_equal(p.ids, cl.perm)
    return p, cl


def compare_sets(p, cl, q, r):
    rowptr, cols = ab.radius_query_csr(p, q, r)
    orp, ocols, _ = oracle.radius_lists(cl, q, r)
    assert np.array_equal(rowptr, orp)
    for i in range(len(q)):
        a = np.sort(cols[rowptr[i]:rowptr[i + 1]])
        b = np.sort(ocols[orp[i]:orp[i + 1]])
        assert np.array_equal(a, b), f"query {i}"


def test_cfg1_counts_and_sets():
    pos = workloads.uniform(100000, 3, seed=11)
    p, cl = build(pos, [0] * 3, [1] * 3, [False] * 3)
    q = p.positions
    counts = ab.radius_count(p, q, 0.05)
    assert np.array_equal(counts, oracle.radius_count(cl, q, 0.05))
    assert 45 < counts.mean() < 56  # ~50.5 neighbours incl. self
    compare_sets(p, cl, q[:3000], 0.05)


@pytest.mark.parametrize("case", KATS["random_brute_force"]["cases"])
def test_reference_random_cases(case):
    d = case["dim"]
    pos = workloads.float_uniform(case["N"], d, seed=99 + d)
    lo, hi = [-1.0] * d, [1.0] * d
    p, cl = build(pos, lo, hi, [case["periodic"]] * d, case["n_leaf"])
    counts = ab.radius_count(p, p.positions, case["r"])
    brute = oracle.brute_counts(p.positions, lo, hi, case["periodic"], case["r"])
    assert np.array_equal(counts, brute)
    compare_sets(p, cl, p.positions, case["r"])


def gauss_circle(r):
    return 1 + 4 * sum(int(math.floor(r ** 2 / (4 * i + 1))) - int(math.floor(r ** 2 / (4 * i + 3)))
                       for i in range(100))


@pytest.mark.parametrize("case", KATS["regular_lattice_l2"]["cases"])
def test_regular_lattice(case):
    d, n = case["dim"], case["n"]
    pos = workloads.lattice(n, d)
    p, cl = build(pos, [0.0] * d, [float(n)] * d, [True] * d, case["n_leaf"])
    counts = ab.radius_count(p, p.positions, case["r"])
    assert np.all(counts == gauss_circle(case["r"]))


def test_mixture_periodic_counts():
    pos = workloads.gaussian_mixture(300000, 3, seed=12)
    p, cl = build(pos, [0] * 3, [1] * 3, [True] * 3)
    q = p.positions
    counts = ab.radius_count(p, q, 0.02)
    sample = np.random.default_rng(0).choice(len(q), 20000, replace=False)
    assert np.array_equal(counts[sample], oracle.radius_count(cl, q[sample], 0.02))
    compare_sets(p, cl, q[sample[:500]], 0.02)


def test_foreign_queries_inside_and_outside():
    pos = workloads.uniform(20000, 3, seed=13)
    for periodic in (False, True):
        p, cl = build(pos, [0] * 3, [1] * 3, [periodic] * 3)
        q = workloads.uniform(5000, 3, lo=-0.2, hi=1.2, seed=14)
        q[:10] = [[5.0, 5.0, 5.0]] * 10
        counts = ab.radius_count(p, q, 0.07)
        assert np.array_equal(counts, oracle.radius_count(cl, q, 0.07))
        compare_sets(p, cl, q[:800], 0.07)


def test_boundary_pairs_exact():
    # points on an exact lattice of spacing 1/16: many pairs at exactly r
    g = (np.arange(16) + 0.5) / 16.0
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    for r in (1 / 16, 2 / 16, np.sqrt(2) / 16, np.sqrt(5) / 16, 0.2):
        for periodic in (False, True):
            p, cl = build(pos, [0] * 3, [1] * 3, [periodic] * 3, 3.0)
            counts = ab.radius_count(p, p.positions, r)
            assert np.array_equal(counts, oracle.radius_count(cl, p.positions, r)), (r, periodic)


def test_large_radius_multiple_images():
    pos = workloads.uniform(300, 2, seed=15)
    p, cl = build(pos, [0, 0], [1, 1], [True, True], 5.0)
    for r in (0.45, 0.6, 0.9):
        counts = ab.radius_count(p, p.positions, r)
        assert np.array_equal(counts, oracle.radius_count(cl, p.positions, r))
        brute = oracle.brute_counts(p.positions, [0, 0], [1, 1], True, r)
        assert np.array_equal(counts, brute)


def test_empty_queries_and_zero_radius():
    pos = workloads.uniform(1000, 3, seed=16)
    p, cl = build(pos, [0] * 3, [1] * 3, [False] * 3)
    assert ab.radius_count(p, np.zeros((0, 3)), 0.1).shape == (0,)
    counts = ab.radius_count(p, p.positions, 0.0)
    assert np.all(counts == 1)


@pytest.mark.parametrize("dim,r", [(3, 0.07), (2, 0.45)])
def test_dx_of_the_accepted_image(dim, r):
    """dx = x_j - (x + image*L) for the periodic image the search accepted,
    bit-exact against the oracle's search iterator (src/Search.h:188-190,
    443); at r = 0.45 in 2-D a particle is often reached through two images,
    each with its own dx."""
    pos = workloads.uniform(4000 if dim == 3 else 600, dim, seed=18)
    p, cl = build(pos, [0] * dim, [1] * dim, [True] * dim, 5.0)
    q = workloads.uniform(300, dim, lo=-0.1, hi=1.1, seed=19)
    rowptr, cols, dx = ab.radius_query_csr(p, q, r, with_dx=True)
    orp, ocols, odx = oracle.radius_lists(cl, q, r, with_dx=True)
    assert np.array_equal(rowptr, orp)
    for i in range(len(q)):
        s = slice(rowptr[i], rowptr[i + 1])
        a = sorted(zip(cols[s].tolist(), map(tuple, dx[s].tolist())))
        b = sorted(zip(ocols[s].tolist(), map(tuple, odx[s].tolist())))
        assert a == b, i
