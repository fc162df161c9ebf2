"""k-nearest neighbours and exact least-squares SPAI rows on the GPU.

The exact rows restate CardinalFunctionsPreconditioner::factorize
(src/Preconditioners.h:1025-1082) on a 32-NN support; they are checked against
numpy's least-squares solution of the same system.
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import workloads

pytestmark = pytest.mark.gpu


def brute_knn(P, k, periodic=False):
    dx = P[:, None, :] - P[None, :, :]
    if periodic:
        dx = dx - np.round(dx)
    d2 = (dx ** 2).sum(-1)
    n = len(P)
    order = np.lexsort((np.broadcast_to(np.arange(n), (n, n)), d2), axis=1)
    return order[:, :k], np.take_along_axis(d2, order[:, :k], 1)


@pytest.mark.parametrize("dim,periodic", [(2, False), (3, False), (2, True)])
def test_knn_vs_brute_force(dim, periodic):
    pos = workloads.uniform(3000, dim, seed=80 + dim)
    p = ab.Particles(dim).set(pos)
    p.init_octree([0.0] * dim, [1.0] * dim, [periodic] * dim, 64)
    idx, d2 = ab.knn(p, 32)
    bi, bd = brute_knn(p.positions, 32, periodic)
    assert np.allclose(d2, bd, rtol=1e-12, atol=1e-15)
    assert np.array_equal(idx, bi)


def test_knn_clustered():
    pos = workloads.gaussian_mixture(5000, 2, k=8, sigma=0.05, seed=84, periodic=False)
    pos = np.clip(pos, 0, 0.999999)
    p = ab.Particles(2).set(pos)
    p.init_octree([0, 0], [1, 1], [False, False], 64)
    idx, d2 = ab.knn(p, 32)
    bi, bd = brute_knn(p.positions, 32)
    assert np.array_equal(idx, bi)


def dense_kernel(P, r, eps2):
    d2 = ((P[:, None, :] - P[None, :, :]) ** 2).sum(-1)
    return np.where(d2 < r * r, np.exp(-d2 * eps2), 0.0)


def test_exact_rows_vs_numpy_lstsq():
    n, eh = 3000, 0.5
    pos = workloads.uniform(n, 2, seed=85)
    eps = eh * np.sqrt(n)
    r = 4.0 / eps
    p = ab.Particles(2).set(pos)
    p.init_octree([0, 0], [1, 1], [False, False], 64)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps))
    cols, vals = ab.spai_exact_rows(K, 32)
    A = dense_kernel(p.positions, r, eps * eps)
    rng = np.random.default_rng(86)
    for i in rng.choice(n, 40, replace=False):
        S = cols[i]
        assert S[0] == i
        U = np.flatnonzero(np.any(A[S] != 0.0, axis=0))
        B = A[np.ix_(U, S)]
        e = (U == i).astype(float)
        w = np.linalg.lstsq(B, e, rcond=None)[0]
        assert np.linalg.norm(vals[i] - w) / np.linalg.norm(w) < 1e-6, i


def test_exact_spai_preconditions_gmres():
    # eps*h = 1: the truncated Gaussian is still positive definite (cond ~1e6)
    n, eh = 20000, 1.0
    pos = workloads.uniform(n, 2, seed=87)
    eps = eh * np.sqrt(n)
    r = 4.0 / eps
    p = ab.Particles(2).set(pos)
    p.init_octree([0, 0], [1, 1], [False, False], 256)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps))
    cols, vals = ab.spai_exact_rows(K, 32)
    M = ab.spai_preconditioner(p.ctx, cols, vals)
    b = np.random.default_rng(88).standard_normal(n)
    _, it_plain, res_plain = ab.gmres(K, b, restart=100, max_iters=400, tol=1e-8)
    x, it, res = ab.gmres(K, b, M=M, restart=100, max_iters=400, tol=1e-8)
    assert res <= 1e-8
    assert it < it_plain


@pytest.mark.parametrize("eh", [2.5, 1.0])
def test_local_inverse_rows_vs_numpy(eh):
    """Local mode (one warp per row): the row solves the k x k system of its
    own k-NN support, A(S, S) w = e_0 -- the exact rows of the learned
    preconditioner.  Against numpy's least-squares solution of the same
    system on sampled rows, including rows next to a near-coincident point
    (eps*h = 1: the local matrices are ill-conditioned, so the check there is
    the residual of the system rather than the weights)."""
    n = 3000
    pos = workloads.uniform(n, 2, seed=89)
    eps = eh * np.sqrt(n)
    r = 4.0 / eps
    p = ab.Particles(2).set(pos)
    p.init_octree([0, 0], [1, 1], [False, False], 64)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps))
    cols, vals = ab.spai_local_inverse_rows(K, 32)
    A = dense_kernel(p.positions, r, eps * eps)
    rng = np.random.default_rng(90)
    for i in rng.choice(n, 60, replace=False):
        S = cols[i]
        assert S[0] == i
        B = A[np.ix_(S, S)]
        e = (S == i).astype(float)
        w = np.linalg.lstsq(B, e, rcond=None)[0]
        res = np.linalg.norm(B @ vals[i] - e)
        assert res <= 1e-9 * max(1.0, np.linalg.norm(vals[i])), (i, res)
        if np.linalg.cond(B) < 1e8:
            assert np.linalg.norm(vals[i] - w) / np.linalg.norm(w) < 1e-8, i
