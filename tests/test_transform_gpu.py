"""Searches in a linearly transformed coordinate system (the reference's
LinearTransform / ScaleTransform, src/Transform.h, applied in the search
iterator as m_dx = transform(p - x), src/Search.h:438-445).

* the known answers of tests/neighbours.h helper_single_particle: one
  particle at the origin of a periodic [-1,1]^3, a scale transform 1/radius
  and max distance 1: one neighbour from (r/2, r/2, 0), none from (2r, 0, 0);
* random particles, a skew transform (the documentation's x + 0.3 y) and an
  anisotropic scale, periodic and not: neighbour sets and transformed dx
  bit-exact against an FP64 brute force over the periodic images with the
  same arithmetic (y = ((T_i0 dx_0 + T_i1 dx_1) + T_i2 dx_2), inside iff
  !(((0 + y_0^2) + y_1^2) + y_2^2 > r^2)).
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import workloads

pytestmark = pytest.mark.gpu


def test_reference_scale_transform_single_particle():
    radius = 0.1
    p = ab.Particles(3).set(np.zeros((1, 3)))
    p.init_neighbour_search([-1.0] * 3, [1.0] * 3, [True] * 3)
    T = np.diag([1.0 / radius] * 3)
    rp, cols, _ = ab.radius_query_csr_transform(p, np.array([[radius / 2, radius / 2, 0.0]]), 1.0, T)
    assert rp[-1] == 1 and cols[0] == 0
    rp, _, _ = ab.radius_query_csr_transform(p, np.array([[2 * radius, 0.0, 0.0]]), 1.0, T)
    assert rp[-1] == 0


def _brute(P, q, r, T, lo, hi, periodic):
    D = P.shape[1]
    L = np.asarray(hi) - np.asarray(lo)
    images = [np.zeros(D)]
    if periodic:
        g = np.array(np.meshgrid(*[[-1, 0, 1]] * D, indexing="ij")).reshape(D, -1).T
        images = [im.astype(float) for im in g]
    out = []
    for x in q:
        found = {}
        for im in images:
            cur = x + im * L
            dx = P - cur
            y = np.zeros_like(dx)
            for i in range(D):
                v = np.zeros(len(P))
                for k in range(D):
                    v = v + T[i, k] * dx[:, k]
                y[:, i] = v
            acc = np.zeros(len(P))
            for i in range(D):
                acc = acc + y[:, i] * y[:, i]
            for j in np.flatnonzero(~(acc > r * r)):
                found[int(j)] = y[j]
        out.append(found)
    return out


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("which", ["skew", "scale"])
def test_transformed_search_vs_brute_force(periodic, which):
    pos = workloads.uniform(20000, 3, seed=240)
    lo, hi = [0.0] * 3, [1.0] * 3
    p = ab.Particles(3).set(pos)
    p.init_neighbour_search(lo, hi, [periodic] * 3, 10.0)
    if which == "skew":
        T = np.array([[1.0, 0.3, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    else:
        T = np.diag([1.0 / 0.02, 1.0 / 0.05, 1.0 / 0.03])
    r = 0.05 if which == "skew" else 1.0
    q = np.concatenate([p.positions[:300], workloads.uniform(100, 3, lo=-0.05, hi=1.05, seed=241)])
    rp, cols, dx = ab.radius_query_csr_transform(p, q, r, T)
    ref = _brute(p.positions, q, r, T, lo, hi, periodic)
    assert sum(len(f) for f in ref) > 1000
    for i in range(len(q)):
        got = {int(c): dx[e] for e, c in zip(range(rp[i], rp[i + 1]), cols[rp[i]:rp[i + 1]])}
        assert set(got) == set(ref[i]), i
        for j, y in got.items():
            assert np.array_equal(y, ref[i][j]), (i, j)


def test_singular_transform_is_rejected():
    p = ab.Particles(2).set(workloads.uniform(100, 2, seed=242))
    p.init_neighbour_search([0, 0], [1, 1], [False, False])
    with pytest.raises(ab.ABXError):
        ab.radius_query_csr_transform(p, p.positions, 0.1, np.array([[1.0, 1.0], [1.0, 1.0]]))
