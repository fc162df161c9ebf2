"""The learned preconditioner's MLP on the GPU: gradients vs the FP64 oracle,
BF16 tensor-core inference vs FP32, training, the learned preconditioner's
gain over no preconditioning, and the Schwarz fallback."""
from pathlib import Path

import numpy as np
import pytest

import aboria_gb300 as ab
import mlp_oracle
import workloads

pytestmark = pytest.mark.gpu
MODEL = Path(__file__).resolve().parent.parent / "aboria_gb300" / "models" / "spai_mlp_2d.bin"


def small_model(seed=91):
    m = ab.MLP.create(64, 128, 3, 32, seed=seed)
    sc = np.linspace(0.5, 2.0, 32).astype(np.float32)
    sh = np.linspace(-0.3, 0.3, 32).astype(np.float32)
    m.set_normalization(1.0, sc, sh)
    return m, sc, sh


def test_gradients_match_oracle():
    m, sc, sh = small_model()
    rng = np.random.default_rng(92)
    x = rng.standard_normal((300, 64)).astype(np.float32)
    y = rng.standard_normal((300, 32)).astype(np.float32)
    loss, g = m.gradients(x, y)
    dims = [64, 128, 128, 128, 32]
    lo, go = mlp_oracle.loss_and_grad(m.params.astype(np.float64), dims, x, y, sc, sh)
    assert abs(loss - lo) / lo < 1e-4
    assert np.linalg.norm(g - go) / np.linalg.norm(go) < 1e-4


def test_bf16_inference_matches_fp32():
    m, sc, sh = small_model(93)
    x = np.random.default_rng(94).standard_normal((1000, 64)).astype(np.float32)
    y32 = m.forward(x, ab.PREC_FP64)
    y16 = m.forward(x, ab.PREC_MIXED)
    ref = mlp_oracle.predict(m.params.astype(np.float64), [64, 128, 128, 128, 32], x, sc, sh)
    assert np.linalg.norm(y32 - ref) / np.linalg.norm(ref) < 1e-5
    assert np.linalg.norm(y16 - ref) / np.linalg.norm(ref) < 2e-2


def test_training_reduces_loss():
    m, _, _ = small_model(95)
    rng = np.random.default_rng(96)
    x = rng.standard_normal((4096, 64)).astype(np.float32)
    W = rng.standard_normal((64, 32)).astype(np.float32) / 8
    y = np.tanh(x @ W).astype(np.float32)
    first = m.train_step(x, y, 1e-3)
    for _ in range(200):
        last = m.train_step(x, y, 1e-3)
    assert last < 0.2 * first


def test_save_load_roundtrip(tmp_path):
    m, _, _ = small_model(97)
    x = np.random.default_rng(98).standard_normal((50, 64)).astype(np.float32)
    path = tmp_path / "m.bin"
    m.save(path)
    m2 = ab.MLP.load(path)
    assert np.array_equal(m.params, m2.params)
    assert np.array_equal(m.forward(x, ab.PREC_FP64), m2.forward(x, ab.PREC_FP64))


def rbf_problem(n, eh, seed):
    pos = workloads.uniform(n, 2, seed=seed)
    eps = eh * np.sqrt(n)
    r = 4.0 / eps
    p = ab.Particles(2).set(pos)
    p.init_octree([0, 0], [1, 1], [False, False], 256)
    K = ab.create_sparse_operator(p, p, r, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps))
    return p, K, eps


@pytest.mark.skipif(not MODEL.exists(), reason="trained model not present")
def test_learned_preconditioner_gain():
    p, K, eps = rbf_problem(50000, 1.2, seed=99)  # test seed, disjoint from training
    m = ab.MLP.load(MODEL)
    M = ab.learned_preconditioner(K, m, eps)
    b = np.random.default_rng(100).standard_normal(len(p))
    _, it0, r0 = ab.gmres(K, b, restart=100, max_iters=600, tol=1e-8)
    x, it1, r1 = ab.gmres(K, b, M=M, restart=100, max_iters=600, tol=1e-8)
    assert r1 <= 1e-8
    assert it1 < it0 / 2, (it0, it1)
    # close to the exact least-squares rows it was trained on
    cols, vals = ab.spai_exact_rows(K, 32)
    lc, lv = ab.spai_rows(M)
    assert np.array_equal(cols, lc)
    assert np.linalg.norm(lv - vals) / np.linalg.norm(vals) < 0.5


def test_fallback_taken_when_learned_fails():
    p, K, eps = rbf_problem(20000, 1.0, seed=101)
    bad = ab.MLP.create(64, 128, 3, 32, seed=5)
    bad.set_normalization(1.0, np.zeros(32, np.float32), np.zeros(32, np.float32))  # M = 0
    Mbad = ab.learned_preconditioner(K, bad, eps)
    b = np.random.default_rng(102).standard_normal(len(p))
    x, it, res, fb = ab.gmres_with_fallback(K, b, Mbad, K, learned_max_iters=50, tol=1e-8)
    assert fb and res <= 1e-8
    r = b - K * x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.0001e-8
