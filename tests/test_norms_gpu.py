"""manhatten_search and chebyshev_search (src/Search.h:797-845) on the GPU:
the radius search in the norms of distance_helper<1> and <-1>
(src/detail/Distance.h:46-137), bit-exact against the oracle's restatement,
and the reference's periodic-lattice box-search known answers
(tests/neighbours.h:679-685: (2 floor(r) + 1)^D neighbours per point)."""
import json
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


def compare(p, cl, q, r, lnorm, nsets=None):
    counts = ab.radius_count(p, q, r, lnorm=lnorm)
    assert np.array_equal(counts, oracle.radius_count(cl, q, r, lnorm=lnorm))
    qs = q if nsets is None else q[:nsets]
    rowptr, cols = ab.radius_query_csr(p, qs, r, lnorm=lnorm)
    orp, ocols, _ = oracle.radius_lists(cl, qs, r, lnorm=lnorm)
    assert np.array_equal(rowptr, orp)
    for i in range(len(qs)):
        assert np.array_equal(np.sort(cols[rowptr[i]:rowptr[i + 1]]),
                              np.sort(ocols[orp[i]:orp[i + 1]])), i
    return counts


@pytest.mark.parametrize("lnorm", [1, -1])
@pytest.mark.parametrize("periodic", [False, True])
def test_uniform_3d(lnorm, periodic):
    pos = workloads.uniform(60000, 3, seed=210)
    p, cl = build(pos, [0] * 3, [1] * 3, [periodic] * 3)
    counts = compare(p, cl, p.positions, 0.06, lnorm, nsets=2000)
    assert counts.min() >= 1


@pytest.mark.parametrize("lnorm", [1, -1])
def test_mixture_and_low_dimensions(lnorm):
    pos = workloads.gaussian_mixture(100000, 3, seed=211)
    p, cl = build(pos, [0] * 3, [1] * 3, [True] * 3)
    compare(p, cl, p.positions[:20000], 0.02, lnorm, nsets=500)
    for dim in (1, 2):
        pos = workloads.uniform(20000, dim, seed=212 + dim)
        p, cl = build(pos, [0] * dim, [1] * dim, [True] * dim)
        compare(p, cl, p.positions, 0.01 if dim == 1 else 0.03, lnorm, nsets=500)


@pytest.mark.parametrize("lnorm", [1, -1])
def test_foreign_queries_and_large_radius(lnorm):
    pos = workloads.uniform(3000, 2, seed=215)
    p, cl = build(pos, [0, 0], [1, 1], [True, True], 5.0)
    q = workloads.uniform(500, 2, lo=-0.3, hi=1.3, seed=216)
    for r in (0.1, 0.45, 0.7):
        compare(p, cl, q, r, lnorm)


@pytest.mark.parametrize("lnorm", [1, -1])
def test_exact_boundary_lattice(lnorm):
    g = (np.arange(12) + 0.5) / 12.0
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    for r in (1 / 12, 2 / 12, 3 / 12):
        for periodic in (False, True):
            p, cl = build(pos, [0] * 3, [1] * 3, [periodic] * 3, 3.0)
            compare(p, cl, p.positions, r, lnorm)


@pytest.mark.parametrize("case", KATS["regular_lattice_linf"]["cases"])
def test_reference_lattice_box_counts(case):
    d, n = case["dim"], case["n"]
    pos = workloads.lattice(n, d)
    p, cl = build(pos, [0.0] * d, [float(n)] * d, [True] * d, case["n_leaf"])
    counts = ab.radius_count(p, p.positions, case["r"], lnorm=-1)
    assert np.all(counts == (2 * int(np.floor(case["r"])) + 1) ** d)


def test_invalid_norm_is_rejected():
    pos = workloads.uniform(100, 3, seed=217)
    p, _ = build(pos, [0] * 3, [1] * 3, [False] * 3)
    with pytest.raises(ab.ABXError):
        ab.radius_count(p, p.positions, 0.1, lnorm=3)
