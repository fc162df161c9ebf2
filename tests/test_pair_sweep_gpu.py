"""Every pair within r once -- the neighbouring-bucket pair sweep of the
reference (bucket_pair_iterator / get_neighbouring_buckets,
src/Search.h:498-764, with the same-bucket pairs; tests/neighbours.h counts
neighbours through it).  Against an FP64 brute force over the periodic
images: the pair set, i < j, the accepted image's dx bit-exact; and the
reference test's use: incrementing both ends of every pair, plus the
particle itself, gives the radius-search counts.
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,periodic", [(3, False), (3, True), (2, True)])
def test_pairs_vs_brute_force(dim, periodic):
    n = 6000
    pos = workloads.uniform(n, dim, seed=250 + dim)
    lo, hi = [0.0] * dim, [1.0] * dim
    p = ab.Particles(dim).set(pos)
    p.init_neighbour_search(lo, hi, [periodic] * dim, 10.0)
    r = 0.06 if dim == 3 else 0.02
    i, j, dx = ab.radius_pairs(p, r)
    assert np.all(i < j) and np.all(np.diff(i) >= 0)
    P = p.positions
    images = [np.zeros(dim)]
    if periodic:
        g = np.array(np.meshgrid(*[[-1, 0, 1]] * dim, indexing="ij")).reshape(dim, -1).T
        images = [im.astype(float) for im in g]
    ref = {}
    for a in range(n):
        for im in images:
            cur = P[a] + im * (np.asarray(hi) - np.asarray(lo))
            d = P[a + 1:] - cur
            acc = np.zeros(len(d))
            for e in range(dim):
                acc = acc + d[:, e] * d[:, e]
            for b in np.flatnonzero(~(acc > r * r)):
                ref[(a, a + 1 + int(b))] = d[b]
    got = {(int(a), int(b)): dx[k] for k, (a, b) in enumerate(zip(i, j))}
    assert len(got) == len(i)
    assert set(got) == set(ref)
    for key, v in got.items():
        assert np.array_equal(v, ref[key]), key
    counts = np.ones(n, dtype=np.int64)
    np.add.at(counts, i, 1)
    np.add.at(counts, j, 1)
    assert np.array_equal(counts, ab.radius_count(p, P, r))
