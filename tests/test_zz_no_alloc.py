"""abx_operator_matvec_noalloc: the sparse matvec for callers that cannot
allocate device memory while applying an operator (a device-memory budget
owned by another runtime, or a loop that cannot afford cudaMalloc's implicit
synchronisation).  It must give the same result as abx_operator_matvec, call
after call, using only the library's fixed scratch array.

Kept in its own file so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import aboria_gb300 as ab
from aboria_gb300 import _lib
import workloads

pytestmark = pytest.mark.gpu
FP64_TOL = 1e-12
MIXED_TOL = 2e-6
ABX_ERR_INVALID, ABX_ERR_STATE, ABX_ERR_CAPACITY = 1, 4, 6


def _noalloc(K, b_dev, c_dev):
    return _lib.lib().abx_operator_matvec_noalloc(K._h, C.c_void_p(b_dev.data_ptr()),
                                                  C.c_void_p(c_dev.data_ptr()))


def _setup(n=300000, seed=41):
    torch = pytest.importorskip("torch")
    pos = workloads.gaussian_mixture(n, 3, seed=seed)
    p = ab.Particles(3).set(pos)
    p.init_neighbour_search([0] * 3, [1] * 3, [True] * 3)
    b = torch.from_numpy(np.random.default_rng(seed + 1).standard_normal(len(p))).cuda()
    return torch, p, b


@pytest.mark.parametrize("prec,tol", [(ab.PREC_FP64, FP64_TOL), (ab.PREC_MIXED, MIXED_TOL)])
def test_noalloc_matches_matvec_twice(prec, tol):
    torch, p, b = _setup()
    r = 0.03
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r), prec)
    ref = K.matvec(b).cpu().numpy()
    for call in range(2):
        c = torch.full_like(b, float("nan"))
        assert _noalloc(K, b, c) == 0, _lib.lib().abx_last_error()
        K.rows.ctx.synchronize()
        got = c.cpu().numpy()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < tol, (call, err)
    # a different right-hand side on the same scratch: no stale contents
    b2 = torch.flip(b, [0]).contiguous()
    ref2 = K.matvec(b2).cpu().numpy()
    c = torch.empty_like(b)
    assert _noalloc(K, b2, c) == 0
    K.rows.ctx.synchronize()
    assert np.linalg.norm(c.cpu().numpy() - ref2) / np.linalg.norm(ref2) < tol


def test_noalloc_rejects_host_vectors_and_oversize():
    torch, p, b = _setup(n=50000, seed=43)
    K = ab.create_sparse_operator(p, p, 0.05, ab.Kernel.make(ab.K_GAUSSIAN, 1600.0))
    bh = np.ones(len(p))
    ch = np.empty(len(p))
    st = _lib.lib().abx_operator_matvec_noalloc(K._h, C.c_void_p(bh.ctypes.data),
                                                C.c_void_p(ch.ctypes.data))
    assert st == ABX_ERR_INVALID
    assert b"device memory" in _lib.lib().abx_last_error()
    # 3M particles need 8 + 8 B each, 48 MB of scratch, in FP64 mode (> 32 MiB)
    big = ab.Particles(3).set(workloads.uniform(3_000_000, 3, seed=44))
    big.init_neighbour_search([0] * 3, [1] * 3, [False] * 3)
    Kb = ab.create_sparse_operator(big, big, 0.005, ab.Kernel.make(ab.K_CONST, 1.0))
    bb = torch.ones(len(big), dtype=torch.float64, device="cuda")
    cb = torch.empty_like(bb)
    assert _noalloc(Kb, bb, cb) == ABX_ERR_CAPACITY
    assert b"scratch" in _lib.lib().abx_last_error()


def test_noalloc_refuses_a_stale_layout_until_rebuilt():
    """After the particle set is searched again the operator's layout is stale;
    rebuilding it would allocate, so the entry point refuses (ABX_ERR_STATE)
    until a regular matvec has rebuilt it."""
    torch, p, b = _setup(n=60000, seed=45)
    r = 0.04
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_WENDLAND_C2, 1 / r), ab.PREC_FP64)
    ref = K.matvec(b).cpu().numpy()
    c = torch.empty_like(b)
    assert _noalloc(K, b, c) == 0
    p.init_neighbour_search([0] * 3, [1] * 3, [True] * 3)
    assert _noalloc(K, b, c) == ABX_ERR_STATE
    assert b"changed" in _lib.lib().abx_last_error()
    K.matvec(b)
    assert _noalloc(K, b, c) == 0
    K.rows.ctx.synchronize()
    assert np.linalg.norm(c.cpu().numpy() - ref) / np.linalg.norm(ref) < FP64_TOL
