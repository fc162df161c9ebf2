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
MODEL3 = MODEL.with_name("spai_mlp_3d.bin")


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
def test_trained_network_gain_over_the_method_without_it():
    """What the trained network gains, on a test instance (seed disjoint from
    training).  The method without it: the same hybrid approximate inverse
    (exact FP64 local-inverse rows next to close neighbours, phi > 0.5) with
    identity rows where the network would answer.  With the network the
    mixed-precision GMRES reaches the FP64-checked 1e-8 in well under 70% of
    the iterations (measured: 13 vs 27), and each network row's residual on its
    own support, |A_i m_i - e_0|, is far below the identity row's."""
    p, K, eps = rbf_problem(50000, 2.5, seed=99)
    K32 = ab.create_sparse_operator(p, p, 4.0 / eps, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps),
                                    ab.PREC_MIXED)
    trained = ab.MLP.load(MODEL)
    ident = ab.MLP.load(MODEL)
    ident.params = np.zeros(ident.num_params, np.float32)  # m = e_0 on every network row
    b = np.random.default_rng(100).standard_normal(len(p))
    Mt = ab.learned_preconditioner(K32, trained, eps)
    Mi = ab.learned_preconditioner(K32, ident, eps)
    assert Mt.stats()["domains"] == Mi.stats()["domains"] > 0
    x, it_t, res_t = ab.gmres(K32, b, M=Mt, restart=100, max_iters=1000, tol=1e-8, A_check=K)
    _, it_i, res_i = ab.gmres(K32, b, M=Mi, restart=100, max_iters=1000, tol=1e-8, A_check=K)
    assert res_t <= 1e-8 and res_i <= 1e-8
    assert it_t < 0.7 * it_i, (it_t, it_i)
    r = b - K * x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.0001e-8
    # per-row residual on the support, network rows only
    idx, d2 = ab.knn(p, 32)
    feats = ab.spai_features(p, idx, eps)
    easy = np.exp(-eps * eps * d2[:, 1]) <= 0.5
    _, vals = ab.spai_rows(Mt)
    A = mlp_oracle.local_matrices(feats[easy], 32, 2, lambda d2_: np.exp(-d2_), 4.0)
    e0 = np.zeros(32)
    e0[0] = 1.0
    res_net = np.linalg.norm(np.einsum("bac,bc->ba", A, vals[easy]) - e0, axis=1)
    res_id = np.linalg.norm(A[:, :, 0] - e0, axis=1)
    assert np.median(res_net) < 0.3 * np.median(res_id), (np.median(res_net), np.median(res_id))
    # the rows next to a close neighbour are the exact local-inverse rows
    cols_x, vals_x = ab.spai_local_inverse_rows(K, 32)
    cols_t, _ = ab.spai_rows(Mt)
    assert np.array_equal(cols_t, cols_x) and np.array_equal(cols_t, idx)
    assert np.array_equal(vals[~easy], vals_x[~easy])
    assert (~easy).sum() == Mt.stats()["domains"]


@pytest.mark.skipif(not MODEL.exists(), reason="trained model not present")
def test_model_on_another_context_gives_the_same_rows():
    """The model and the operator may live on different contexts (streams) of
    one device: the library orders the inference between them, so the rows
    are bit-identical to the same-context ones."""
    p, K, eps = rbf_problem(40000, 2.5, seed=103)
    same = ab.MLP.load(MODEL, ctx=p.ctx)
    other = ab.MLP.load(MODEL, ctx=ab.Context(0))
    _, v_same = ab.spai_rows(ab.learned_preconditioner(K, same, eps))
    for _ in range(3):
        _, v_other = ab.spai_rows(ab.learned_preconditioner(K, other, eps))
        assert np.array_equal(v_same, v_other)


@pytest.mark.skipif(not MODEL3.exists(), reason="trained model not present")
def test_trained_3d_network_gain():
    """The 3-D model on a 3-D test instance: the hybrid approximate inverse with
    the network reaches 1e-8 (FP64-checked) in under 60% of the iterations of
    the same method with identity rows (measured 8 vs 22 at N=50,000)."""
    n, eh = 30000, 2.5
    pos = workloads.uniform(n, 3, seed=199)
    eps = eh * n ** (1 / 3)
    p = ab.Particles(3).set(pos)
    p.init_octree([0] * 3, [1] * 3, [False] * 3, 256)
    kern = ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps)
    K64 = ab.create_sparse_operator(p, p, 4 / eps, kern)
    K32 = ab.create_sparse_operator(p, p, 4 / eps, kern, ab.PREC_MIXED)
    trained = ab.MLP.load(MODEL3)
    ident = ab.MLP.load(MODEL3)
    ident.params = np.zeros(ident.num_params, np.float32)
    b = np.random.default_rng(200).standard_normal(n)
    _, it_t, res_t = ab.gmres(K32, b, M=ab.learned_preconditioner(K32, trained, eps), restart=100,
                              max_iters=1000, tol=1e-8, A_check=K64)
    _, it_i, res_i = ab.gmres(K32, b, M=ab.learned_preconditioner(K32, ident, eps), restart=100,
                              max_iters=1000, tol=1e-8, A_check=K64)
    assert res_t <= 1e-8 and res_i <= 1e-8
    assert it_t < 0.6 * it_i, (it_t, it_i)


def test_fallback_taken_when_learned_fails():
    p, K, eps = rbf_problem(20000, 2.0, seed=101)
    bad = ab.MLP.create(64, 128, 3, 32, seed=5)
    bad.set_normalization(1.0, np.zeros(32, np.float32), np.zeros(32, np.float32))  # M = 0
    Mbad = ab.learned_preconditioner(K, bad, eps, exact_phi=1.0)  # every row from the network
    b = np.random.default_rng(102).standard_normal(len(p))
    x, it, res, fb = ab.gmres_with_fallback(K, b, Mbad, K, learned_max_iters=50, tol=1e-8)
    assert fb and res <= 1e-8
    r = b - K * x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.0001e-8
