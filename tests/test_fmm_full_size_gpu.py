"""Chebyshev black-box FMM at the FMM benchmark's sizes (3-D, uniform in the
unit cube, Laplace 1/(|dx| + 1e-12), octree leaves of 64, weights U[-1,1]).

The self term K(0) b_i = 1e12 b_i is taken out of both sides: the FMM result
minus 1e12 b_i against a direct sum that skips j == i (summed with the self
term inside, the direct sum would round ~1e-4 off every later term, an error
of the same size as the order-7 interpolation error).

* N = 1,048,576, orders 3/5/7, FP64 and mixed (3xTF32 tensor-core M2L, FP32
  P2P) modes, against the oracle's FP64 direct sum on 10,000 seeded targets
  (relative L2).  Tolerances are the Chebyshev interpolation error of each
  order with a margin; the mixed mode may add at most 1e-5 on top of FP64.
* N = 16,777,216, order 5, mixed, against the oracle's FP64 direct sum on
  1,000 seeded targets.
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu

LAPLACE = [1e-12]
TOL = {3: 3e-3, 5: 1e-4, 7: 3e-5}


def _tree(n, seed):
    pos = workloads.uniform(n, 3, seed=seed)
    p = ab.Particles(3).set(pos)
    p.init_octree([0.0] * 3, [1.0] * 3, [False] * 3, 64)
    return p


def _err(K, b, tgt, direct):
    c = (K * b)[tgt] - 1e12 * b[tgt]
    return np.linalg.norm(c - direct) / np.linalg.norm(direct)


@pytest.fixture(scope="module")
def n1m():
    n = 1 << 20
    p = _tree(n, 5050)
    b = np.random.default_rng(5051).uniform(-1, 1, n)
    tgt = np.sort(np.random.default_rng(5052).choice(n, 10_000, replace=False))
    direct = oracle.direct_sum(p.positions, ab.K_LAPLACE, LAPLACE, b, tgt, skip_self=True)
    return p, b, tgt, direct


@pytest.mark.parametrize("order", [3, 5, 7])
def test_fmm_1m_vs_oracle_direct_sum(n1m, order):
    p, b, tgt, direct = n1m
    K = ab.create_fmm_operator(p, ab.Kernel.make(ab.K_LAPLACE, *LAPLACE), order)
    e64 = _err(K, b, tgt, direct)
    K.set_precision(ab.PREC_MIXED)
    e32 = _err(K, b, tgt, direct)
    assert e64 < TOL[order], e64
    assert e32 < e64 + 1e-5, (e32, e64)


def test_fmm_16m_order5_mixed_vs_oracle_direct_sum():
    n = 1 << 24
    p = _tree(n, 6060)
    b = np.random.default_rng(6061).uniform(-1, 1, n)
    tgt = np.sort(np.random.default_rng(6062).choice(n, 1_000, replace=False))
    direct = oracle.direct_sum(p.positions, ab.K_LAPLACE, LAPLACE, b, tgt, skip_self=True)
    K = ab.create_fmm_operator(p, ab.Kernel.make(ab.K_LAPLACE, *LAPLACE), 5)
    K.set_precision(ab.PREC_MIXED)
    e32 = _err(K, b, tgt, direct)
    assert e32 < TOL[5], e32
