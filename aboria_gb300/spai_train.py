"""Train the learned sparse-approximate-inverse model on the GPU.

Training data: exact FP64 Schwarz block-solve rows on the 32-nearest-neighbour
domain of each particle (``abx_spai_local_inverse_rows``: row i of the local
block inverse), of compactly supported Gaussian RBF operators
exp(-(eps |dx|)^2), cut where the
Gaussian has decayed to e^-16 (r = 4/eps), on seeded training instances:
2-D point sets, uniform or an 8-component Gaussian mixture (sigma 0.05), with
the scaled shape parameter eps*h drawn uniform on [2, 3] (h = N^-1/2 the mean
spacing).  Below eps*h ~ 0.75 the truncated Gaussian matrix is indefinite or
numerically singular and no preconditioner reaches 1e-8; between ~0.75 and 2
its local inverses have weights up to 1e5 (near-coincident points) and a
sparse approximate inverse stops working once its weights carry ~0.3% error,
which no regression reaches.  The least-squares rows
(``abx_spai_exact_rows``) depend on geometry beyond the 32 neighbours the
features describe, so they are not used as labels.  Rows whose weights exceed
1e3 in magnitude are dropped.  Instance seeds start at 1000, disjoint from every test seed.
Features are the 32 neighbours' relative positions scaled by eps; targets are
the 32 weights w, trained as asinh(w / c) (c the median |w|, which compresses
the heavy tails of ill-conditioned rows) normalised per output by mean and
standard deviation; inference applies the inverse, c * sinh(.).

The network (3 hidden layers of 128, SiLU) is trained with the library's own
forward/backward/Adam kernels (``abx_mlp_train_step``) and saved with
``abx_mlp_save``.

    python -m aboria_gb300.spai_train --out aboria_gb300/models/spai_mlp_2d.bin
"""
from __future__ import annotations

import argparse
import time

import numpy as np

import aboria_gb300 as ab

K = 32


def instance(seed, n, dim=2):
    rng = np.random.default_rng(seed)
    if rng.uniform() < 0.5:
        pos = rng.uniform(0.0, 1.0, size=(n, dim))
    else:
        centres = rng.uniform(0.15, 0.85, size=(8, dim))
        pos = centres[rng.integers(0, 8, size=n)] + 0.05 * rng.standard_normal((n, dim))
        pos = np.clip(pos, 0.0, np.nextafter(1.0, 0.0))
    eh = rng.uniform(2.0, 3.0)
    eps = eh * np.sqrt(n)
    return pos, eps


def make_rows(seed, n, dim=2):
    pos, eps = instance(seed, n, dim)
    p = ab.Particles(dim).set(pos)
    p.init_octree([0.0] * dim, [1.0] * dim, [False] * dim, 256)
    op = ab.create_sparse_operator(p, p, 4.0 / eps, ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps))
    cols, vals = ab.spai_local_inverse_rows(op, K)
    feats = ab.spai_features(p, cols, eps)
    return feats, vals.astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--instances", type=int, default=40)
    ap.add_argument("--n", type=int, default=50000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    args = ap.parse_args()
    t0 = time.time()
    X, Y = [], []
    for i in range(args.instances):
        f, v = make_rows(1000 + i, args.n)
        X.append(f)
        Y.append(v)
    X = np.concatenate(X)
    Y = np.concatenate(Y)
    ok = np.all(np.isfinite(Y), axis=1) & (np.abs(Y).max(axis=1) < 1e3)
    X, Y = X[ok], Y[ok]
    print(f"rows {len(X)} (dropped {int((~ok).sum())}) in {time.time() - t0:.1f}s", flush=True)
    # compress the heavy tails: train on asinh(w / c), infer c * sinh(.)
    c = float(np.median(np.abs(Y)))
    T = np.arcsinh(Y / c).astype(np.float32)
    shift = T.mean(axis=0).astype(np.float32)
    scale = np.maximum(T.std(axis=0), 1e-6).astype(np.float32)
    m = ab.MLP.create(X.shape[1], 128, 3, K, seed=7)
    m.set_normalization(1.0, scale, shift)
    m.set_output_transform(1, c)
    Y = T
    import torch
    Xd = torch.from_numpy(X).cuda()
    Yd = torch.from_numpy(Y).cuda()
    rng = np.random.default_rng(3)
    steps = 0
    nb = len(X) // args.batch
    t1 = time.time()
    for ep in range(args.epochs):
        lr = args.lr * (0.5 * (1 + np.cos(np.pi * ep / args.epochs)))
        perm = torch.from_numpy(rng.permutation(len(X))).cuda()
        tot = 0.0
        for b in range(nb):
            idx = perm[b * args.batch:(b + 1) * args.batch]
            xb = Xd[idx].contiguous()
            yb = Yd[idx].contiguous()
            tot += m.train_step(xb, yb, lr)
            steps += 1
        print(f"epoch {ep} loss {tot / nb:.5f} lr {lr:.2e}", flush=True)
    print(f"trained {steps} steps in {time.time() - t1:.1f}s", flush=True)
    m.save(args.out)


if __name__ == "__main__":
    main()
