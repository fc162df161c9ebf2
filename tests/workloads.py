"""Seeded synthetic particle workloads with the shapes of the benchmark configs."""
import numpy as np


def uniform(n, dim=3, lo=0.0, hi=1.0, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=(n, dim))


def float_uniform(n, dim, seed):
    """Uniform in [-1,1]^D drawn in float32, as the reference's random tests."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, size=(n, dim)).astype(np.float32).astype(np.float64)


def gaussian_mixture(n, dim=3, k=16, sigma=0.03, frac_uniform=0.2, seed=0, periodic=True):
    """k isotropic Gaussians (centres U[0.1,0.9]^D) + a uniform background,
    wrapped into the periodic unit box."""
    rng = np.random.default_rng(seed)
    nu = int(round(frac_uniform * n))
    nc = n - nu
    centres = rng.uniform(0.1, 0.9, size=(k, dim))
    which = rng.integers(0, k, size=nc)
    pts = centres[which] + sigma * rng.standard_normal((nc, dim))
    bg = rng.uniform(0.0, 1.0, size=(nu, dim))
    x = np.concatenate([pts, bg])
    x = x[rng.permutation(n)]
    if periodic:
        x = np.mod(x, 1.0)
        x[x >= 1.0] = 0.0
    return x


def lattice(n, dim):
    """n^dim lattice points at (i + 1/2), index 0 fastest (tests/neighbours.h:640-660)."""
    idx = np.stack(np.meshgrid(*[np.arange(n)] * dim, indexing="ij"), -1).reshape(-1, dim)
    idx = idx[:, ::-1]
    return idx.astype(np.float64) + 0.5


def clipped_mixture(n, dim, k=8, sigma=0.05, seed=0):
    """k isotropic Gaussians (centres U[0.15,0.85]^D, sigma 0.05) clipped into
    the unit box: the clustered point sets of the RBF-solve grid."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.15, 0.85, size=(k, dim))
    pts = centres[rng.integers(0, k, size=n)] + sigma * rng.standard_normal((n, dim))
    return np.clip(pts, 0.0, np.nextafter(1.0, 0.0))
