"""Black-box Chebyshev FMM on the GPU.

* FP64 mode vs the oracle's restatement of the reference FMM (same tree,
  traversal and expansions; the oracle evaluates M2L kernels on the fly as
  the reference does): 1e-10 relative.
* The reference's FMM known-answer test (tests/fmm.h:167-253) through the GPU.
* Laplace 1/(|dx| + 1e-12) accuracy vs an FP64 direct sum, FP64 and mixed
  (3xTF32 tensor-core M2L, FP32 P2P) modes; the self term K(0) b_i is removed
  before comparing so that it does not hide the approximation error.
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu


def octree(pos, n_leaf):
    d = pos.shape[1]
    p = ab.Particles(d).set(pos)
    p.init_octree([0.0] * d, [1.0] * d, [False] * d, n_leaf)
    return p


@pytest.mark.parametrize("dim,order", [(3, 3), (3, 5), (2, 4)])
def test_fmm_fp64_matches_oracle(dim, order):
    n = 4000 if dim == 3 else 6000
    pos = workloads.uniform(n, dim, seed=120 + order)
    p = octree(pos, 32)
    b = np.random.default_rng(121).uniform(-1, 1, n)
    K = ab.create_fmm_operator(p, ab.Kernel.make(ab.K_MULTIQUADRIC, 0.01), order)
    c = K * b
    ref = oracle.fmm(p.positions, [0.0] * dim, [1.0] * dim, 32, order, ab.K_MULTIQUADRIC, [0.01], b)
    assert np.linalg.norm(c - ref) / np.linalg.norm(ref) < 1e-10


@pytest.mark.parametrize("dim", [2, 3])
def test_reference_fmm_kat(dim):
    N = 1000
    pos = workloads.uniform(N, dim, seed=130 + dim)
    p = octree(pos, 10)
    P = p.positions
    b = np.prod(np.cos(2 * np.pi * P), axis=1) / N
    direct = oracle.direct_sum(P, ab.K_MULTIQUADRIC, [0.01], b, np.arange(N))
    K = ab.create_fmm_operator(p, ab.Kernel.make(ab.K_MULTIQUADRIC, 0.01), 3)
    c = K * b
    assert np.sum((c - direct) ** 2) / np.sum(direct ** 2) < 1e-2


@pytest.mark.parametrize("order,tol64", [(3, 3e-2), (5, 2e-3), (7, 2e-4)])
def test_laplace_vs_direct_sum(order, tol64):
    n = 100000
    pos = workloads.uniform(n, 3, seed=140)
    p = octree(pos, 64)
    P = p.positions
    b = np.random.default_rng(141).uniform(-1, 1, n)
    kern = ab.Kernel.make(ab.K_LAPLACE, 1e-12)
    targets = np.random.default_rng(142).choice(n, 1000, replace=False)
    direct = oracle.direct_sum(P, ab.K_LAPLACE, [1e-12], b, targets) - 1e12 * b[targets]
    K = ab.create_fmm_operator(p, kern, order)
    c64 = (K * b)[targets] - 1e12 * b[targets]
    e64 = np.linalg.norm(c64 - direct) / np.linalg.norm(direct)
    assert e64 < tol64, e64
    K.set_precision(ab.PREC_MIXED)
    c32 = (K * b)[targets] - 1e12 * b[targets]
    e32 = np.linalg.norm(c32 - direct) / np.linalg.norm(direct)
    assert e32 < tol64 * 1.5 + 1e-5, (e32, e64)


@pytest.mark.parametrize("order", [4, 5, 6, 7, 8])
def test_mixed_m2l_matches_fp64_for_every_row_block_count(order):
    """Mixed mode against FP64 mode on the same tree, self term removed.
    Orders 5..8 (125..512 Chebyshev nodes) run the tcgen05 M2L with 1..4 row
    blocks of 128 per CTA; order 4 runs the mma.sync M2L.  A row block or a
    split part that went missing would show as an error of order 1 or 1e-3."""
    n = 30000
    pos = workloads.uniform(n, 3, seed=150 + order)
    p = octree(pos, 64)
    b = np.random.default_rng(151 + order).uniform(-1, 1, n)
    K = ab.create_fmm_operator(p, ab.Kernel.make(ab.K_LAPLACE, 1e-12), order)
    c64 = K * b - 1e12 * b
    K.set_precision(ab.PREC_MIXED)
    c32 = K * b - 1e12 * b
    assert ab.fmm_stats(K)["m2l_pairs"] > 0
    err = np.linalg.norm(c32 - c64) / np.linalg.norm(c64)
    assert err < 1e-5, err


def test_m2l_wait_timeout_is_reported_and_the_context_survives():
    """The tensor-core M2L bounds every mbarrier wait by the GPU's global
    timer.  With one operand-ready signal withheld (a barrier nothing arrives
    on) the MMA issuer's wait runs out: the matvec must return ABX_ERR_TIMEOUT
    after the kernel drained its copies and freed its tensor memory, and the
    next matvec on the same context must be correct."""
    n = 30000
    pos = workloads.uniform(n, 3, seed=170)
    p = octree(pos, 64)
    b = np.random.default_rng(171).uniform(-1, 1, n)
    K = ab.create_fmm_operator(p, ab.Kernel.make(ab.K_LAPLACE, 1e-12), 5)
    c64 = K * b - 1e12 * b
    K.set_precision(ab.PREC_MIXED)
    ab.fmm_set_wait_limit(K, 0.02, drop_one_arrive=True)
    with pytest.raises(ab.ABXError) as exc:
        K * b
    assert exc.value.status == 5  # ABX_ERR_TIMEOUT
    ab.fmm_set_wait_limit(K, 1.0, drop_one_arrive=False)
    for _ in range(2):
        c32 = K * b - 1e12 * b
        assert np.linalg.norm(c32 - c64) / np.linalg.norm(c64) < 1e-5
