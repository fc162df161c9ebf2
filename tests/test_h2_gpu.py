"""The H2 operator (create_h2_operator, src/Operators.h:440-447; H2Matrix,
src/H2Matrix.h:46-110): the black-box Chebyshev plan with the admissibility
parameter eta, built once and reused by every K*b.

* eta = 1 is the FMM's admissibility rule: the H2 and FMM operators of one
  octree have the same M2L pairs and agree in FP64 to rounding (the M2L
  adds into the local expansions with atomics, in no fixed order).
* A pair of boxes is far (M2L) when their gap is at least max diameter / eta:
  a smaller eta keeps more pairs near (P2P, or refined to the next level),
  and the error against the oracle's FP64 direct sum does not grow.
* The kernel of the reference's H2 tests (tests/h2.h:407-420), the
  multiquadric sqrt(|dx|^2 + 0.001), at order 4, FP64 and mixed precision.
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu


def _tree(n, seed):
    p = ab.Particles(3).set(workloads.uniform(n, 3, seed=seed))
    p.init_octree([0.0] * 3, [1.0] * 3, [False] * 3, 32)
    return p


def test_h2_eta1_equals_fmm():
    p = _tree(20000, 300)
    b = np.random.default_rng(301).uniform(-1, 1, len(p))
    k = ab.Kernel.make(ab.K_MULTIQUADRIC, 0.001)
    F = ab.create_fmm_operator(p, k, 4)
    H = ab.create_h2_operator(p, k, 4, eta=1.0)
    cf, ch = F * b, H * b
    assert np.linalg.norm(cf - ch) / np.linalg.norm(cf) < 1e-13
    assert ab.fmm_stats(F)["m2l_pairs"] == ab.fmm_stats(H)["m2l_pairs"]


def test_h2_eta_trades_work_for_accuracy():
    p = _tree(20000, 302)
    P = p.positions
    b = np.random.default_rng(303).uniform(-1, 1, len(p))
    k = ab.Kernel.make(ab.K_MULTIQUADRIC, 0.001)
    tgt = np.random.default_rng(304).choice(len(p), 2000, replace=False)
    direct = oracle.direct_sum(P, ab.K_MULTIQUADRIC, [0.001], b, tgt)
    errs, pairs = [], []
    for eta in (1.0, 0.75, 0.5):
        H = ab.create_h2_operator(p, k, 4, eta=eta)
        c = (H * b)[tgt]
        errs.append(np.linalg.norm(c - direct) / np.linalg.norm(direct))
        pairs.append(ab.fmm_stats(H)["m2l_pairs"])
        H.set_precision(ab.PREC_MIXED)
        c32 = (H * b)[tgt]
        assert np.linalg.norm(c32 - direct) / np.linalg.norm(direct) < errs[-1] + 1e-5
    assert pairs[2] != pairs[0], pairs
    assert errs[2] <= errs[1] * 1.05 and errs[1] <= errs[0] * 1.05, errs
    assert errs[2] < errs[0], errs
    assert errs[0] < 1e-3, errs


def test_h2_rejects_bad_eta():
    p = _tree(2000, 305)
    with pytest.raises(ab.ABXError):
        ab.create_h2_operator(p, ab.Kernel.make(ab.K_LAPLACE, 1e-12), 3, eta=0.0)
