"""Train the learned sparse-approximate-inverse model on the GPU.

Model: the 32 nearest neighbours' positions relative to the row's point,
scaled by the shape parameter eps (32 x dim features), -> MLP (3 hidden
layers of 128, SiLU) -> the row's 32 weights as m = e_0 + 0.1 y, a correction
to the identity row.

Loss (ABX_LOSS_SPAI_RESIDUAL): the approximate-inverse residual of each row on
its own support, |A_i m_i - e_0|^2, with A_i the 32 x 32 compactly supported
Gaussian matrix exp(-|f_a - f_b|^2) (zero for |f_a - f_b| >= 4, i.e. the
operator's cut-off eps |dx| < 4) of the row's support points, built from the
features themselves.  Its minimiser is the exact FP64 local-inverse row (the
Schwarz block solve on the 32-NN domain, abx_spai_local_inverse_rows), and
|A_i m - e_0|^2 = |A_i (m - m*)|^2: the distance to that label measured in
the metric of the local matrix.  A plain weight MSE spends the network's
capacity on weight directions the matrix barely sees (large, cancelling
weights next to near-coincident points) and its rows failed to precondition.

Rows: only rows whose nearest other point has phi = exp(-(eps d)^2) <= 0.5;
the preconditioner solves the other rows exactly (exact_phi = 0.5).

Instances: 2-D or 3-D (--dim), uniform or an 8-component Gaussian mixture
(sigma 0.05), the scaled shape parameter eps*h uniform on [--eh-lo, --eh-hi]
(h = N^(-1/dim); default [1, 3]), instance seeds from 1000 (disjoint from
every test seed).
Below eps*h ~ 0.75 the truncated Gaussian matrix is numerically singular and
no preconditioner reaches 1e-8.

The committed models were trained with the defaults (eps*h in [1, 3]):

    python -m aboria_gb300.spai_train --out aboria_gb300/models/spai_mlp_2d.bin
    python -m aboria_gb300.spai_train --dim 3 --out aboria_gb300/models/spai_mlp_3d.bin
"""
from __future__ import annotations

import argparse
import time

import numpy as np

import aboria_gb300 as ab

K = 32
EXACT_PHI = 0.5


def instance(seed, n, dim=2, eh_range=(1.0, 3.0)):
    rng = np.random.default_rng(seed)
    if rng.uniform() < 0.5:
        pos = rng.uniform(0.0, 1.0, size=(n, dim))
    else:
        centres = rng.uniform(0.15, 0.85, size=(8, dim))
        pos = centres[rng.integers(0, 8, size=n)] + 0.05 * rng.standard_normal((n, dim))
        pos = np.clip(pos, 0.0, np.nextafter(1.0, 0.0))
    eh = rng.uniform(*eh_range)
    eps = eh * n ** (1.0 / dim)
    return pos, eps


def easy_rows(seed, n, dim=2, eh_range=(1.0, 3.0)):
    """Features of the rows the network serves (phi of the nearest other point <= EXACT_PHI)."""
    pos, eps = instance(seed, n, dim, eh_range)
    p = ab.Particles(dim).set(pos)
    p.init_octree([0.0] * dim, [1.0] * dim, [False] * dim, 256)
    idx, d2 = ab.knn(p, K)
    feats = ab.spai_features(p, idx, eps)
    phi_nn = np.exp(-eps * eps * d2[:, 1])
    return feats[phi_nn <= EXACT_PHI]


def make_model(seed=7, dim=2):
    m = ab.MLP.create(K * dim, 128, 3, K, seed=seed)
    shift = np.zeros(K, np.float32)
    shift[0] = 1.0
    m.set_normalization(1.0, np.full(K, 0.1, np.float32), shift)
    m.set_loss(ab.LOSS_SPAI_RESIDUAL, dim, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, 1.0), 4.0)
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--dim", type=int, default=2)
    ap.add_argument("--instances", type=int, default=40)
    ap.add_argument("--n", type=int, default=50000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eh-lo", type=float, default=1.0)
    ap.add_argument("--eh-hi", type=float, default=3.0)
    args = ap.parse_args()
    t0 = time.time()
    X = np.concatenate([easy_rows(1000 + i, args.n, args.dim, (args.eh_lo, args.eh_hi))
                        for i in range(args.instances)])
    print(f"rows {len(X)} in {time.time() - t0:.1f}s", flush=True)
    m = make_model(dim=args.dim)
    import torch
    Xd = torch.from_numpy(X).cuda()
    rng = np.random.default_rng(3)
    steps = 0
    nb = len(X) // args.batch
    t1 = time.time()
    for ep in range(args.epochs):
        lr = args.lr * (0.5 * (1 + np.cos(np.pi * ep / args.epochs)))
        perm = torch.from_numpy(rng.permutation(len(X))).cuda()
        tot = 0.0
        for b in range(nb):
            xb = Xd[perm[b * args.batch:(b + 1) * args.batch]].contiguous()
            tot += m.train_step(xb, None, lr)
            steps += 1
        print(f"epoch {ep} residual {tot / nb:.5f} lr {lr:.2e}", flush=True)
    print(f"trained {steps} steps in {time.time() - t1:.1f}s", flush=True)
    m.save(args.out)


if __name__ == "__main__":
    main()
