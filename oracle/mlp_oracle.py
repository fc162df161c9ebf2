"""FP64 numpy restatement of the learned preconditioner's MLP (TEST
INFRASTRUCTURE ONLY): same flat parameter layout (per layer W [in x out]
row-major then b [out]), SiLU hidden activations, linear output, and the two
training losses: mean squared error on normalised targets, and the
approximate-inverse residual mean_i |A_i m_i - e_0|^2 with A_i the kernel
matrix of row i's support points read from its features.  Used to check the
GPU's hand-written forward, backward and Adam kernels."""
import numpy as np


def unpack(params, dims):
    Ws, bs, o = [], [], 0
    for l in range(len(dims) - 1):
        a, b = dims[l], dims[l + 1]
        Ws.append(params[o:o + a * b].reshape(a, b))
        o += a * b
        bs.append(params[o:o + b])
        o += b
    return Ws, bs


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, dims, x, in_scale=1.0):
    Ws, bs = unpack(np.asarray(params, np.float64), dims)
    a = np.asarray(x, np.float64) * in_scale
    acts, pres = [a], []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = a @ W + b
        pres.append(z)
        a = silu(z) if l < len(Ws) - 1 else z
        acts.append(a)
    return acts, pres


def loss_and_grad(params, dims, x, y, out_scale, out_shift, in_scale=1.0):
    acts, pres = forward(params, dims, x, in_scale)
    t = (np.asarray(y, np.float64) - out_shift) / out_scale
    out = acts[-1]
    n = out.size
    loss = np.sum((out - t) ** 2) / n
    d = 2.0 * (out - t) / n
    return loss, _backward(params, dims, acts, pres, d)


def local_matrices(x, k, dim, kern, cutoff=0.0):
    """A[b, a, c] = kern(|f_c - f_a|^2) inside the cut-off (features f, k points)."""
    f = np.asarray(x, np.float64).reshape(-1, k, dim)
    d2 = ((f[:, :, None, :] - f[:, None, :, :]) ** 2).sum(-1)
    A = kern(d2)
    if cutoff > 0:
        A = np.where(d2 < cutoff * cutoff, A, 0.0)
    return A


def residual_loss_and_grad(params, dims, x, dim, kern, cutoff, out_scale, out_shift,
                           in_scale=1.0):
    """Loss mean_i |A_i m_i - e_0|^2 (m_i = out_i * scale + shift) and its gradient."""
    acts, pres = forward(params, dims, x, in_scale)
    out = acts[-1]
    B, k = out.shape
    m = out * out_scale + out_shift
    A = local_matrices(x, k, dim, kern, cutoff)
    r = np.einsum("bac,bc->ba", A, m)
    r[:, 0] -= 1.0
    loss = np.sum(r ** 2) / B
    d = out_scale * 2.0 * np.einsum("bac,bc->ba", A, r) / B
    return loss, _backward(params, dims, acts, pres, d)


def _backward(params, dims, acts, pres, d):
    Ws, _ = unpack(np.asarray(params, np.float64), dims)
    grads = []
    for l in range(len(Ws) - 1, -1, -1):
        if l < len(Ws) - 1:
            d = d * silu_grad(pres[l])
        gW = acts[l].T @ d
        gb = d.sum(0)
        grads.append((gW, gb))
        if l > 0:
            d = d @ Ws[l].T
    flat = []
    for gW, gb in reversed(grads):
        flat.append(gW.ravel())
        flat.append(gb)
    return np.concatenate(flat)


def predict(params, dims, x, out_scale, out_shift, in_scale=1.0):
    acts, _ = forward(params, dims, x, in_scale)
    return acts[-1] * out_scale + out_shift
