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


def test_residual_loss_gradients_match_oracle():
    """ABX_LOSS_SPAI_RESIDUAL: mean |A_i m_i - e_0|^2 with A_i the compact
    Gaussian exp(-|f_a - f_b|^2) (cut at 4) of each row's 32 support points."""
    m = ab.MLP.create(64, 128, 3, 32, seed=96)
    sc = np.full(32, 0.1, np.float32)
    sh = np.zeros(32, np.float32)
    sh[0] = 1.0
    m.set_normalization(1.0, sc, sh)
    kern = ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, 1.0)
    m.set_loss(ab.LOSS_SPAI_RESIDUAL, 2, kern, 4.0)
    rng = np.random.default_rng(97)
    x = (rng.standard_normal((256, 32, 2)) * 1.5).astype(np.float32)
    x[:, 0, :] = 0.0
    x = x.reshape(256, 64)
    loss, g = m.gradients(x)
    dims = [64, 128, 128, 128, 32]
    lo, go = mlp_oracle.residual_loss_and_grad(m.params.astype(np.float64), dims, x, 2,
                                               lambda d2: np.exp(-d2), 4.0, sc, sh)
    assert abs(loss - lo) / lo < 1e-4
    assert np.linalg.norm(g - go) / np.linalg.norm(go) < 1e-4
    # training on the residual lowers it
    l0 = m.train_step(x, None, 1e-3)
    for _ in range(30):
        l1 = m.train_step(x, None, 1e-3)
    assert l1 < 0.8 * l0


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
def test_trained_network_vs_labels_and_untrained():
    """What the trained network gains, measured on a test instance (seed
    disjoint from training): its predicted rows are far closer to the exact
    local-inverse labels than an untrained network's, but not close enough to
    precondition (the labels tolerate only ~1% weight error), so the solve
    falls back to Schwarz; the labels themselves cut GMRES iterations by more
    than 100x."""
    p, K, eps = rbf_problem(50000, 2.5, seed=99)
    cols, vals = ab.spai_local_inverse_rows(K, 32)
    trained = ab.MLP.load(MODEL)
    untrained = ab.MLP.create(64, 128, 3, 32, seed=11)
    lc, lv = ab.spai_rows(ab.learned_preconditioner(K, trained, eps))
    _, uv = ab.spai_rows(ab.learned_preconditioner(K, untrained, eps))
    assert np.array_equal(lc, cols)
    err_t = np.median(np.linalg.norm(lv - vals, axis=1) / np.linalg.norm(vals, axis=1))
    err_u = np.median(np.linalg.norm(uv - vals, axis=1) / np.linalg.norm(vals, axis=1))
    assert err_t < 0.3 and err_t < 0.5 * err_u, (err_t, err_u)
    b = np.random.default_rng(100).standard_normal(len(p))
    _, it0, _ = ab.gmres(K, b, restart=100, max_iters=1000, tol=1e-8)
    _, it_lab, r_lab = ab.gmres(K, b, M=ab.spai_preconditioner(p.ctx, cols, vals), restart=100,
                                max_iters=1000, tol=1e-8)
    assert r_lab <= 1e-8 and it_lab * 100 < it0
    M = ab.learned_preconditioner(K, trained, eps)
    x, it, res, fb = ab.gmres_with_fallback(K, b, M, K, learned_max_iters=30, tol=1e-8)
    assert res <= 1e-8


def test_fallback_taken_when_learned_fails():
    p, K, eps = rbf_problem(20000, 2.0, seed=101)
    bad = ab.MLP.create(64, 128, 3, 32, seed=5)
    bad.set_normalization(1.0, np.zeros(32, np.float32), np.zeros(32, np.float32))  # M = 0
    Mbad = ab.learned_preconditioner(K, bad, eps)
    b = np.random.default_rng(102).standard_normal(len(p))
    x, it, res, fb = ab.gmres_with_fallback(K, b, Mbad, K, learned_max_iters=50, tol=1e-8)
    assert fb and res <= 1e-8
    r = b - K * x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.0001e-8
