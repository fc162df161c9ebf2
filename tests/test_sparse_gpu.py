"""GPU sparse and dense operators vs the oracle.

FP64 mode: the reference's arithmetic (FP64 radius test, FP64 kernel values
and accumulation); parity bar 1e-12 relative (L2 norm) against the oracle,
which sums in the reference's neighbour order.
Mixed mode: FP32 kernel values, FP32 blocks of <=32 terms summed in FP64;
its error against FP64 is asserted below 2e-6 relative (L2) -- the stated
tolerance of the mixed-precision path.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())
FP64_TOL = 1e-12
MIXED_TOL = 2e-6


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def build(pos, lo, hi, periodic, n_leaf=10.0):
    p = ab.Particles(pos.shape[1]).set(pos)
    p.init_neighbour_search(lo, hi, periodic, n_leaf)
    cl = oracle.celllist_build(pos, lo, hi, periodic, n_leaf)
    assert np.array_equal(p.ids, cl.perm)
    return p, cl


def test_sparse_kat():
    k = KATS["sparse_operator"]
    pos = np.array(k["positions"])
    p, cl = build(pos, k["domain_lo"], k["domain_hi"], k["periodic"])
    ids = p.ids
    p.set_scalar(np.full(3, k["scalar1"]))
    q = ab.Particles(3).set(pos)  # the same particles, second scalar column
    q.init_neighbour_search(k["domain_lo"], k["domain_hi"], k["periodic"])
    q.set_scalar(np.full(3, k["scalar2"]))
    C = ab.create_sparse_operator(p, q, k["radius"], ab.Kernel.make(ab.K_SCALAR_SUM))
    v = np.array(k["v"], float)[ids]
    ans = np.empty(3)
    ans[ids] = C * v
    assert list(ans) == k["answer"]
    rowptr, cols = ab.radius_query_csr(q, p.positions, k["radius"])
    assert rowptr[-1] == k["nonzeros"]


def test_dense_kat():
    k = KATS["dense_operator"]
    pos = np.array(k["positions"])
    a = ab.Particles(3).set(pos)
    a.set_scalar(np.full(3, k["scalar1"]))
    b = ab.Particles(3).set(pos)
    b.set_scalar(np.full(3, k["scalar2"]))
    A = ab.create_dense_operator(a, b, ab.Kernel.make(ab.K_SCALAR_SUM))
    for case in k["cases"]:
        assert list(A * np.array(case["v"], float)) == case["answer"]


def test_cfg1_gaussian_fp64_and_mixed():
    r = 0.05
    pos = workloads.uniform(100000, 3, seed=21)
    p, cl = build(pos, [0] * 3, [1] * 3, [False] * 3)
    b = np.random.default_rng(22).uniform(0, 1, len(p))
    kern = ab.Kernel.make(ab.K_GAUSSIAN, 1.0 / (r / 2) ** 2)
    ref = oracle.sparse_matvec(cl, cl.pos, r, ab.K_GAUSSIAN, [1.0 / (r / 2) ** 2], b)
    K = ab.create_sparse_operator(p, p, r, kern)
    assert rel(K * b, ref) < FP64_TOL
    K.set_precision(ab.PREC_MIXED)
    assert rel(K * b, ref) < MIXED_TOL


def test_cfg2_shape_wendland_periodic_reduced():
    r = 0.02
    pos = workloads.gaussian_mixture(400000, 3, seed=23)
    p, cl = build(pos, [0] * 3, [1] * 3, [True] * 3)
    b = np.random.default_rng(24).standard_normal(len(p))
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1.0 / r)
    K = ab.create_sparse_operator(p, p, r, kern)
    c64 = K * b
    sample = np.random.default_rng(25).choice(len(p), 4000, replace=False)
    ref = oracle.sparse_matvec(cl, cl.pos[sample], r, ab.K_WENDLAND_C2, [1.0 / r], b)
    assert rel(c64[sample], ref) < FP64_TOL
    K.set_precision(ab.PREC_MIXED)
    c32 = K * b
    assert rel(c32, c64) < MIXED_TOL


@pytest.mark.parametrize("kind,params", [(ab.K_LAPLACE, [1e-12]), (ab.K_MULTIQUADRIC, [0.01]),
                                         (ab.K_COMPACT_GAUSSIAN, [400.0]), (ab.K_CONST, [2.5])])
def test_other_kernels(kind, params):
    r = 0.08
    pos = workloads.uniform(30000, 2, seed=26)
    p, cl = build(pos, [0, 0], [1, 1], [True, False])
    b = np.random.default_rng(27).standard_normal(len(p))
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(kind, *params))
    ref = oracle.sparse_matvec(cl, cl.pos, r, kind, params, b)
    assert rel(K * b, ref) < FP64_TOL
    K.set_precision(ab.PREC_MIXED)
    assert rel(K * b, ref) < MIXED_TOL


def test_rows_differ_from_cols():
    r = 0.06
    cols_pos = workloads.uniform(30000, 3, seed=28)
    rows_pos = workloads.uniform(7000, 3, lo=-0.05, hi=1.05, seed=29)
    pc, cl = build(cols_pos, [0] * 3, [1] * 3, [True] * 3)
    pr = ab.Particles(3).set(rows_pos)
    pr.init_neighbour_search([-0.05] * 3, [1.05] * 3, [False] * 3)
    b = np.random.default_rng(30).standard_normal(len(pc))
    K = ab.create_sparse_operator(pr, pc, r, ab.Kernel.make(ab.K_GAUSSIAN, 300.0))
    assert K.shape == (len(pr), len(pc))
    ref = oracle.sparse_matvec(cl, pr.positions, r, ab.K_GAUSSIAN, [300.0], b)
    assert rel(K * b, ref) < FP64_TOL


def test_device_vectors_and_linearity():
    torch = pytest.importorskip("torch")
    r = 0.05
    pos = workloads.uniform(50000, 3, seed=31)
    p, cl = build(pos, [0] * 3, [1] * 3, [False] * 3)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r))
    rng = np.random.default_rng(32)
    b1, b2 = rng.standard_normal(len(p)), rng.standard_normal(len(p))
    d1 = torch.from_numpy(b1).cuda()
    c_dev = K * d1
    assert c_dev.is_cuda
    c_host = K * b1
    assert np.array_equal(c_dev.cpu().numpy(), c_host)
    lhs = K * (2.0 * b1 + b2)
    rhs = 2.0 * (K * b1) + (K * b2)
    assert rel(lhs, rhs) < 1e-13


@pytest.mark.parametrize("dim,n", [(3, 3000), (2, 1001)])
def test_dense_vs_oracle(dim, n):
    """FP64 mode bit-for-bit in the reference's column order (1e-14); mixed
    mode (packed FP32x2 pairs, an odd tile tail padded with a zero-weight
    column) to 1e-5."""
    pos = workloads.uniform(n, dim, seed=33)
    a = ab.Particles(dim).set(pos)
    rng = np.random.default_rng(34)
    b = rng.standard_normal(n)
    for kind, params in ((ab.K_GAUSSIAN, [30.0]), (ab.K_MULTIQUADRIC, [0.01]),
                         (ab.K_LAPLACE, [1e-12]), (ab.K_WENDLAND_C2, [5.0])):
        A = ab.create_dense_operator(a, a, ab.Kernel.make(kind, *params))
        ref = oracle.dense_matvec(pos, pos, kind, params, b)
        c = A * b
        # FP64 mode walks the columns in the reference's order
        assert rel(c, ref) < 1e-14, kind
        A.set_precision(ab.PREC_MIXED)
        assert rel(A * b, ref) < 1e-5, kind


def test_empty_operator():
    p = ab.Particles(3).set(np.zeros((0, 3)))
    p.init_neighbour_search([0] * 3, [1] * 3, [False] * 3)
    K = ab.create_sparse_operator(p, p, 0.1, ab.Kernel.make(ab.K_CONST, 1.0))
    assert (K * np.zeros(0)).shape == (0,)


def test_dense_chunked_and_empty_columns():
    """Few rows against many columns: the mixed kernel splits the columns into
    chunks (79 here) whose row sums are added in order; no columns: zeros."""
    rows = workloads.uniform(300, 3, seed=35)
    cols = workloads.uniform(20000, 3, seed=36)
    b = np.random.default_rng(37).standard_normal(20000)
    r, c = ab.Particles(3).set(rows), ab.Particles(3).set(cols)
    A = ab.create_dense_operator(r, c, ab.Kernel.make(ab.K_GAUSSIAN, 30.0), ab.PREC_MIXED)
    ref = oracle.dense_matvec(rows, cols, ab.K_GAUSSIAN, [30.0], b)
    assert rel(A * b, ref) < 1e-5
    assert np.array_equal(A * b, A * b)  # deterministic
    e = ab.Particles(3).set(np.zeros((0, 3)))
    for prec in (ab.PREC_MIXED, ab.PREC_FP64):
        E = ab.create_dense_operator(r, e, ab.Kernel.make(ab.K_GAUSSIAN, 30.0), prec)
        assert np.array_equal(E * np.zeros(0), np.zeros(300))
