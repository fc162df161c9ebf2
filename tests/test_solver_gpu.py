"""Schwarz preconditioner and GMRES on the GPU.

* RAS apply vs the oracle's restatement (same domains, LU with partial
  pivoting): 1e-9 relative (LU rounding differs between the two factorisations).
* GMRES solutions vs a dense FP64 direct solve (numpy) and the true residual.
* The reference's compact RBF interpolation test (tests/rbf_interpolation.h:
  245-416): GMRES-RAS on a Wendland kernel, RMS < 1e-4 at the centres and
  < 1e-2 away from them (no polynomial augmentation here).
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu


def octree_particles(pos, n_leaf, periodic=False):
    d = pos.shape[1]
    p = ab.Particles(d).set(pos)
    p.init_octree([0.0] * d, [1.0] * d, [periodic] * d, n_leaf)
    return p


def dense_matrix(P, r, kind, params, periodic=False):
    dx = P[None, :, :] - P[:, None, :]
    if periodic:
        dx = dx - np.round(dx)
    d2 = (dx ** 2).sum(-1)
    if kind == ab.K_WENDLAND_C2:
        q = np.sqrt(d2) * params[0]
        v = np.where(q < 1, (1 - q) ** 4 * (4 * q + 1), 0.0)
    else:
        v = np.exp(-d2 * params[0])
    return np.where(d2 <= r * r, v, 0.0)


@pytest.mark.parametrize("dim,periodic", [(2, False), (3, False), (2, True)])
def test_schwarz_apply_matches_oracle(dim, periodic):
    n, r = 4000, 0.12 if dim == 2 else 0.2
    pos = workloads.uniform(n, dim, seed=70 + dim)
    p = octree_particles(pos, 64, periodic)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r))
    M = ab.schwarz_preconditioner(K)
    t = oracle.octree_build(pos, [0.0] * dim, [1.0] * dim, 64)
    b = np.random.default_rng(71).standard_normal(n)
    x = M.solve(b)
    ref = oracle.schwarz_apply(p.positions, [0.0] * dim, [1.0] * dim, [periodic] * dim, t, r,
                               ab.K_WENDLAND_C2, [1 / r], b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9
    st = M.stats()
    assert st["domains"] == np.count_nonzero(t.leaf_end > t.leaf_begin)


def test_schwarz_mixed_factors_close():
    n, r = 4000, 0.12
    p = octree_particles(workloads.uniform(n, 2, seed=72), 64)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r))
    b = np.random.default_rng(73).standard_normal(n)
    x64 = ab.schwarz_preconditioner(K).solve(b)
    x32 = ab.schwarz_preconditioner(K, ab.PREC_MIXED).solve(b)
    assert np.linalg.norm(x32 - x64) / np.linalg.norm(x64) < 1e-3


def numpy_gmres(A, b, m, maxit):
    """Textbook restarted GMRES(m) (MGS Arnoldi, least squares per cycle)."""
    x = np.zeros(len(b))
    tot = 0
    while True:
        r = b - A @ x
        beta = np.linalg.norm(r)
        if tot >= maxit:
            return x, beta / np.linalg.norm(b)
        V = [r / beta]
        H = np.zeros((m + 1, m))
        for j in range(m):
            w = A @ V[j]
            for i in range(j + 1):
                H[i, j] = V[i] @ w
                w = w - H[i, j] * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            V.append(w / H[j + 1, j])
            tot += 1
        e = np.zeros(m + 1)
        e[0] = beta
        x = x + np.array(V[:m]).T @ np.linalg.lstsq(H, e, rcond=None)[0]


def test_gmres_matches_textbook_algorithm():
    n, r = 2000, 0.1
    p = octree_particles(workloads.uniform(n, 2, seed=74), 64)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r))
    A = dense_matrix(p.positions, r, ab.K_WENDLAND_C2, [1 / r])
    b = np.random.default_rng(75).standard_normal(n)
    x, it, res = ab.gmres(K, b, restart=50, max_iters=300, tol=1e-14)
    xr, resr = numpy_gmres(A, b, 50, 300)
    assert it == 300
    # CGS2 (GPU) and MGS (numpy) Arnoldi differ only by rounding over 300 steps
    assert abs(res - resr) / resr < 1e-4
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-4


def test_gmres_schwarz_vs_dense_solve():
    n, r = 2000, 0.1
    p = octree_particles(workloads.uniform(n, 2, seed=74), 64)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r))
    A = dense_matrix(p.positions, r, ab.K_WENDLAND_C2, [1 / r])
    b = np.random.default_rng(75).standard_normal(n)
    x, it, res = ab.gmres(K, b, M=ab.schwarz_preconditioner(K), restart=50, max_iters=2000,
                          tol=1e-10)
    assert res <= 1e-10 and it < 200
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-7
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9


def test_mixed_gmres_refined_to_fp64_residual():
    n, r = 20000, 0.08
    p = octree_particles(workloads.uniform(n, 2, seed=76), 128)
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r)
    K64 = ab.create_sparse_operator(p, p, r, kern)
    K32 = ab.create_sparse_operator(p, p, r, kern, ab.PREC_MIXED)
    M = ab.schwarz_preconditioner(K64)
    b = np.random.default_rng(77).standard_normal(n)
    x, it, res = ab.gmres(K32, b, M=M, restart=100, max_iters=3000, tol=1e-8, A_check=K64)
    assert res <= 1e-8, (it, res)
    # each refinement cycle contracts the FP64 residual by about
    # cond(A) * (FP32 operator error) ~ 0.1 for this matrix
    assert it < 400
    r64 = b - K64 * x
    assert np.linalg.norm(r64) / np.linalg.norm(b) <= 1.0001e-8


def test_reference_compact_rbf_interpolation():
    N = 1000
    rng = np.random.default_rng(123)
    knots_pos = rng.uniform(0, 1, (N, 2))
    test_pos = rng.uniform(0, 1, (N, 2))
    f = lambda x, y: np.exp(-9 * (x - 0.5) ** 2 - 9 * (y - 0.25) ** 2)
    h = 4.0 * N ** -0.5
    knots = octree_particles(knots_pos, 50)
    test = ab.Particles(2).set(test_pos)
    test.init_neighbour_search([0, 0], [1, 1], [False, False])
    # (2 - |dx|/h)^4 (1 + 2|dx|/h) = 16 * Wendland C2 with q = |dx|/(2h)
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1 / (2 * h))
    G = ab.create_sparse_operator(knots, knots, 2 * h, kern)
    G_test = ab.create_sparse_operator(test, knots, 2 * h, kern)
    P = knots.positions
    phi = f(P[:, 0], P[:, 1])
    gamma, it, res = ab.gmres(G, phi, M=ab.schwarz_preconditioner(G), restart=101,
                              max_iters=100, tol=1e-12)
    fit = G * gamma
    assert np.sqrt(np.sum((fit - phi) ** 2) / np.sum(phi ** 2)) < 1e-4
    T = test.positions
    truth = f(T[:, 0], T[:, 1])
    ev = G_test * gamma
    assert np.sqrt(np.sum((ev - truth) ** 2) / np.sum(truth ** 2)) < 1e-2
