"""aboria_gb300: the GB300 (sm_103a) particle hot path behind Aboria's API.

Python mirror of the reference's operator interface over the C ABI declared
in ``include/abx.h`` (ctypes, no torch types in the boundary).  Names follow
the reference: ``Particles`` with ``init_neighbour_search``,
``euclidean_search`` counts/lists, ``create_sparse_operator``,
``create_dense_operator`` and ``K * b``.

Vector arguments may be numpy arrays (host memory) or CUDA tensors / any
object exposing ``data_ptr()`` (device memory); the library stages host
buffers itself.  There is no CPU fallback: if the CUDA library cannot be
loaded every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from ._lib import ABXError, closing, lib, load_library  # noqa: F401

__all__ = [
    "ABXError", "Context", "Particles", "Kernel", "Operator", "create_sparse_operator",
    "create_dense_operator", "radius_count", "radius_query_csr", "PREC_FP64", "PREC_MIXED",
    "LOSS_MSE", "LOSS_SPAI_RESIDUAL",
    "K_CONST", "K_GAUSSIAN", "K_WENDLAND_C2", "K_COMPACT_GAUSSIAN", "K_LAPLACE",
    "K_MULTIQUADRIC", "K_SCALAR_SUM", "default_context", "Preconditioner",
    "schwarz_preconditioner", "spai_preconditioner", "gmres", "knn", "spai_exact_rows", "MLP",
    "spai_features", "learned_preconditioner", "spai_local_inverse_rows", "create_fmm_operator", "fmm_stats", "spai_rows", "gmres_with_fallback",
    "fp32_peak_tflops", "fmm_set_wait_limit", "create_h2_operator", "radius_query_csr_transform", "radius_pairs",
]

PREC_FP64, PREC_MIXED = 0, 1
LOSS_MSE, LOSS_SPAI_RESIDUAL = 0, 1
(K_CONST, K_GAUSSIAN, K_WENDLAND_C2, K_COMPACT_GAUSSIAN, K_LAPLACE, K_MULTIQUADRIC,
 K_SCALAR_SUM) = range(7)


def _ptr(a):
    """Raw pointer of a numpy array (host) or a tensor-like (device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return C.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported array type {type(a)!r}")


def _check(status, what="abx call"):
    if status != 0:
        msg = lib().abx_last_error().decode(errors="replace")
        raise ABXError(status, f"{what} failed ({status}): {msg}")


class Context:
    """One device and one stream (``abx_context``)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = C.c_void_p()
        _check(lib().abx_context_create(device, C.c_void_p(stream or 0), C.byref(self._h)),
               "abx_context_create")

    def synchronize(self):
        _check(lib().abx_context_synchronize(self._h), "abx_context_synchronize")

    def close(self):
        if self._h and not closing():
            lib().abx_context_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("ABX_DEVICE", "0")))
    return _default_ctx


class Particles:
    """``Particles<std::tuple<scalar>, D>`` (src/Particles.h:108-112)."""

    def __init__(self, dim: int = 3, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.dim = dim
        self._h = C.c_void_p()
        _check(lib().abx_particles_create(self.ctx._h, dim, C.byref(self._h)),
               "abx_particles_create")

    def __del__(self):
        try:
            if self._h and not closing():
                lib().abx_particles_destroy(self._h)
        except Exception:
            pass

    def __len__(self):
        return int(lib().abx_particles_size(self._h))

    def set(self, pos, ids=None):
        """Replace the contents with ``len(pos)`` particles (like push_back)."""
        n = int(pos.shape[0])
        if isinstance(pos, np.ndarray):
            pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(n, self.dim)
        if ids is not None and isinstance(ids, np.ndarray):
            ids = np.ascontiguousarray(ids, dtype=np.int64)
        _check(lib().abx_particles_set(self._h, n, _ptr(pos), _ptr(ids)), "abx_particles_set")
        return self

    def set_scalar(self, s):
        if isinstance(s, np.ndarray):
            s = np.ascontiguousarray(s, dtype=np.float64)
        _check(lib().abx_particles_set_scalar(self._h, _ptr(s)), "abx_particles_set_scalar")

    def set_positions(self, pos):
        if isinstance(pos, np.ndarray):
            pos = np.ascontiguousarray(pos, dtype=np.float64)
        _check(lib().abx_particles_set_positions(self._h, _ptr(pos)),
               "abx_particles_set_positions")

    def init_neighbour_search(self, lo, hi, periodic, n_particles_in_leaf: float = 10.0):
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        per = np.ascontiguousarray([1 if p else 0 for p in periodic], dtype=np.int32)
        _check(lib().abx_particles_init_neighbour_search(self._h, _ptr(lo), _ptr(hi), _ptr(per),
                                                         float(n_particles_in_leaf)),
               "abx_particles_init_neighbour_search")
        return self

    def init_octree(self, lo, hi, periodic, n_particles_in_leaf: float = 10.0):
        """``Particles<..., HyperOctree>::init_neighbour_search``."""
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        per = np.ascontiguousarray([1 if p else 0 for p in periodic], dtype=np.int32)
        _check(lib().abx_particles_init_octree(self._h, _ptr(lo), _ptr(hi), _ptr(per),
                                               float(n_particles_in_leaf)),
               "abx_particles_init_octree")
        return self

    def tree_leaves(self):
        """Octree leaves: (level, tag, begin, end) arrays in creation order."""
        n = C.c_int64()
        _check(lib().abx_particles_get_tree_leaves(self._h, C.byref(n), None, None, None, None, 0),
               "get_tree_leaves")
        out = [np.empty(n.value, dtype=np.int32) for _ in range(4)]
        _check(lib().abx_particles_get_tree_leaves(self._h, C.byref(n), *map(_ptr, out), n.value),
               "get_tree_leaves")
        return tuple(out)

    def update_positions(self):
        _check(lib().abx_particles_update_positions(self._h), "abx_particles_update_positions")

    def push_back(self, pos):
        """Append particles (``Particles::push_back``); returns their ids.  A
        searchable set is re-searched at once, as the reference does."""
        pos = np.ascontiguousarray(np.atleast_2d(pos), dtype=np.float64).reshape(-1, self.dim)
        ids = np.empty(len(pos), dtype=np.int64)
        _check(lib().abx_particles_push_back(self._h, len(pos), _ptr(pos), _ptr(ids)),
               "abx_particles_push_back")
        return ids

    def erase(self, first: int, last: int | None = None):
        """``Particles::erase``: drop the particles at storage positions
        [first, last) (last defaults to first + 1)."""
        last = first + 1 if last is None else last
        _check(lib().abx_particles_erase(self._h, int(first), int(last)), "abx_particles_erase")

    def find_ids(self, ids):
        """Storage index of every id (-1 where absent): find-by-id."""
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        out = np.empty(len(ids), dtype=np.int64)
        _check(lib().abx_particles_find_ids(self._h, len(ids), _ptr(ids), _ptr(out)),
               "abx_particles_find_ids")
        return out

    @property
    def positions(self) -> np.ndarray:
        out = np.empty((len(self), self.dim), dtype=np.float64)
        _check(lib().abx_particles_get_positions(self._h, _ptr(out)), "get_positions")
        return out

    @property
    def ids(self) -> np.ndarray:
        out = np.empty(len(self), dtype=np.int64)
        _check(lib().abx_particles_get_ids(self._h, _ptr(out)), "get_ids")
        return out

    @property
    def scalar(self) -> np.ndarray:
        out = np.empty(len(self), dtype=np.float64)
        _check(lib().abx_particles_get_scalar(self._h, _ptr(out)), "get_scalar")
        return out

    def grid(self):
        size = np.zeros(self.dim, dtype=np.uint32)
        side = np.zeros(self.dim, dtype=np.float64)
        nc = C.c_uint32()
        _check(lib().abx_particles_get_grid(self._h, _ptr(size), _ptr(side), C.byref(nc)),
               "get_grid")
        return size, side, int(nc.value)

    def buckets(self):
        _, _, nc = self.grid()
        bb = np.empty(nc, dtype=np.uint32)
        be = np.empty(nc, dtype=np.uint32)
        keys = np.empty(len(self), dtype=np.uint32)
        _check(lib().abx_particles_get_buckets(self._h, _ptr(bb), _ptr(be), _ptr(keys)),
               "get_buckets")
        return bb, be, keys


def radius_count(p: Particles, q, r: float, out=None, lnorm: int = 2):
    """Neighbour counts of ``euclidean_search(p.get_query(), q_i, r)``;
    lnorm 1 / -1 give ``manhatten_search`` / ``chebyshev_search``."""
    nq = int(q.shape[0])
    if isinstance(q, np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float64)
    if out is None:
        out = np.empty(nq, dtype=np.int32)
    _check(lib().abx_radius_count_lnorm(p._h, nq, _ptr(q), float(r), int(lnorm), _ptr(out)),
           "abx_radius_count")
    return out


def radius_query_csr(p: Particles, q, r: float, lnorm: int = 2, with_dx: bool = False):
    """Neighbour lists (storage indices) as CSR ``(rowptr, cols)``; lnorm as
    for radius_count.  with_dx (euclidean only) also returns dx[nnz, dim],
    x_j - (x + image*L) for the periodic image the search accepted."""
    nq = int(q.shape[0])
    q = np.ascontiguousarray(q, dtype=np.float64)
    rowptr = np.empty(nq + 1, dtype=np.int64)
    _check(lib().abx_radius_query_csr_lnorm(p._h, nq, _ptr(q), float(r), int(lnorm), _ptr(rowptr),
                                            None, 0), "abx_radius_query_csr")
    nnz = int(rowptr[-1])
    cols = np.empty(max(nnz, 1), dtype=np.int32)
    if with_dx:
        if lnorm != 2:
            raise ValueError("dx is returned by the euclidean search only")
        dx = np.empty((max(nnz, 1), p.dim), dtype=np.float64)
        _check(lib().abx_radius_query_csr_dx(p._h, nq, _ptr(q), float(r), _ptr(rowptr), _ptr(cols),
                                             _ptr(dx), nnz), "abx_radius_query_csr_dx")
        return rowptr, cols[:nnz], dx[:nnz]
    _check(lib().abx_radius_query_csr_lnorm(p._h, nq, _ptr(q), float(r), int(lnorm), _ptr(rowptr),
                                            _ptr(cols), nnz), "abx_radius_query_csr")
    return rowptr, cols[:nnz]


def radius_pairs(p: Particles, r: float):
    """Every pair within r once (the neighbouring-bucket pair sweep):
    ``(i, j, dx)`` with i < j storage indices, dx = x_j - (x_i + image*L)."""
    n = C.c_int64()
    _check(lib().abx_radius_pairs(p._h, float(r), C.byref(n), None, None, None, 0),
           "abx_radius_pairs")
    m = n.value
    i = np.empty(max(m, 1), dtype=np.int32)
    j = np.empty(max(m, 1), dtype=np.int32)
    dx = np.empty((max(m, 1), p.dim), dtype=np.float64)
    _check(lib().abx_radius_pairs(p._h, float(r), C.byref(n), _ptr(i), _ptr(j), _ptr(dx), m),
           "abx_radius_pairs")
    return i[:m], j[:m], dx[:m]


def radius_query_csr_transform(p: Particles, q, r: float, T):
    """``euclidean_search(query, x, r, transform)`` with a linear transform
    (``create_linear_transform`` / ``create_scale_transform``) given as its
    dim x dim matrix T: CSR ``(rowptr, cols, dx)``, dx the transformed
    separations T (x_j - x - image*L) of the neighbours."""
    nq = int(q.shape[0])
    q = np.ascontiguousarray(q, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64).reshape(p.dim, p.dim)
    rowptr = np.empty(nq + 1, dtype=np.int64)
    _check(lib().abx_radius_query_csr_transform(p._h, nq, _ptr(q), float(r), _ptr(T),
                                                _ptr(rowptr), None, None, 0),
           "abx_radius_query_csr_transform")
    nnz = int(rowptr[-1])
    cols = np.empty(max(nnz, 1), dtype=np.int32)
    dx = np.empty((max(nnz, 1), p.dim), dtype=np.float64)
    _check(lib().abx_radius_query_csr_transform(p._h, nq, _ptr(q), float(r), _ptr(T),
                                                _ptr(rowptr), _ptr(cols), _ptr(dx), nnz),
           "abx_radius_query_csr_transform")
    return rowptr, cols[:nnz], dx[:nnz]


class Kernel(C.Structure):
    _fields_ = [("kind", C.c_int), ("p", C.c_double * 4)]

    @classmethod
    def make(cls, kind: int, *params: float) -> "Kernel":
        k = cls()
        k.kind = kind
        for i, v in enumerate(params[:4]):
            k.p[i] = float(v)
        return k


class Operator:
    """``MatrixReplacement``: ``K * b`` returns ``c = K b``."""

    def __init__(self, h, rows: Particles, cols: Particles):
        self._h = h
        self.rows, self.cols = rows, cols  # held by reference, as the reference does

    def __del__(self):
        try:
            if self._h and not closing():
                lib().abx_operator_destroy(self._h)
        except Exception:
            pass

    def set_precision(self, mode: int):
        _check(lib().abx_operator_set_precision(self._h, mode), "set_precision")
        return self

    @property
    def shape(self):
        return (int(lib().abx_operator_rows(self._h)), int(lib().abx_operator_cols(self._h)))

    def matvec(self, b, out=None, sync=True):
        """``c = K b``.  Host (numpy) results are complete on return; device
        results are synchronised with the context stream unless sync=False."""
        nr, nc = self.shape
        if isinstance(b, np.ndarray):
            b = np.ascontiguousarray(b, dtype=np.float64)
            if b.shape[0] != nc:
                raise ValueError(f"rhs has {b.shape[0]} rows, operator has {nc} columns")
            if out is None:
                out = np.empty(nr, dtype=np.float64)
        elif out is None:
            import torch  # device tensors only
            out = torch.empty(nr, dtype=torch.float64, device=b.device)
        _check(lib().abx_operator_matvec(self._h, _ptr(b), _ptr(out)), "abx_operator_matvec")
        if sync and not isinstance(out, np.ndarray):
            self.rows.ctx.synchronize()
        return out

    def __mul__(self, b):
        return self.matvec(b)


def create_sparse_operator(rows: Particles, cols: Particles, radius: float, kernel: Kernel,
                           precision: int = PREC_FP64) -> Operator:
    h = C.c_void_p()
    _check(lib().abx_create_sparse_operator(rows._h, cols._h, float(radius), C.byref(kernel),
                                            C.byref(h)), "abx_create_sparse_operator")
    return Operator(h, rows, cols).set_precision(precision)


def create_dense_operator(rows: Particles, cols: Particles, kernel: Kernel,
                          precision: int = PREC_FP64) -> Operator:
    h = C.c_void_p()
    _check(lib().abx_create_dense_operator(rows._h, cols._h, C.byref(kernel), C.byref(h)),
           "abx_create_dense_operator")
    return Operator(h, rows, cols).set_precision(precision)


class Preconditioner:
    """``x = M b``: SchwartzPreconditioner or a sparse approximate inverse."""

    def __init__(self, h, ctx, n, keep=()):
        self._h = h
        self.ctx = ctx
        self.n = n
        self._keep = keep

    def __del__(self):
        try:
            if self._h and not closing():
                lib().abx_precond_destroy(self._h)
        except Exception:
            pass

    def solve(self, b, out=None):
        if isinstance(b, np.ndarray):
            b = np.ascontiguousarray(b, dtype=np.float64)
            out = np.empty(self.n) if out is None else out
        elif out is None:
            import torch
            out = torch.empty(self.n, dtype=torch.float64, device=b.device)
        _check(lib().abx_precond_apply(self._h, _ptr(b), _ptr(out)), "abx_precond_apply")
        if not isinstance(out, np.ndarray):
            self.ctx.synchronize()
        return out

    def stats(self):
        nd, ms, el = C.c_int64(), C.c_int64(), C.c_int64()
        t = C.c_double()
        _check(lib().abx_precond_stats(self._h, C.byref(nd), C.byref(ms), C.byref(el), C.byref(t)),
               "abx_precond_stats")
        ph = [C.c_double() for _ in range(4)]
        _check(lib().abx_precond_setup_phases(self._h, *[C.byref(x) for x in ph]),
               "abx_precond_setup_phases")
        return {"domains": nd.value, "max_size": ms.value, "elements": el.value,
                "setup_s": t.value, "knn_s": ph[0].value, "features_s": ph[1].value,
                "infer_s": ph[2].value, "exact_rows_s": ph[3].value}


def schwarz_preconditioner(op: Operator, precision: int = PREC_FP64) -> Preconditioner:
    """``SchwartzPreconditioner<LU>``: analyzePattern + factorize on ``op``."""
    h = C.c_void_p()
    _check(lib().abx_precond_create_schwarz(op._h, precision, C.byref(h)),
           "abx_precond_create_schwarz")
    return Preconditioner(h, op.rows.ctx, op.shape[0], keep=(op,))


def spai_preconditioner(ctx: Context, cols, vals) -> Preconditioner:
    """Sparse approximate inverse with ``k`` entries per row (cols, vals: n x k)."""
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    n, k = cols.shape
    h = C.c_void_p()
    _check(lib().abx_precond_create_spai(ctx._h, n, k, _ptr(cols), _ptr(vals), C.byref(h)),
           "abx_precond_create_spai")
    return Preconditioner(h, ctx, n)


def gmres(A: Operator, b, x0=None, M: Preconditioner | None = None, restart: int = 100,
          max_iters: int = 1000, tol: float = 1e-8, A_check: Operator | None = None):
    """Restarted flexible GMRES; returns (x, iterations, relative residual)."""
    n = A.shape[0]
    if isinstance(b, np.ndarray):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    else:
        import torch
        x = torch.zeros(n, dtype=torch.float64, device=b.device) if x0 is None else x0.clone()
    it = C.c_int()
    res = C.c_double()
    _check(lib().abx_gmres_solve(A._h, A_check._h if A_check else None, M._h if M else None,
                                 _ptr(b), _ptr(x), int(restart), int(max_iters), float(tol),
                                 C.byref(it), C.byref(res)), "abx_gmres_solve")
    if not isinstance(x, np.ndarray):
        A.rows.ctx.synchronize()
    return x, it.value, res.value


def knn(p: Particles, k: int = 32):
    """k nearest neighbours of every stored particle: (idx, d2), each n x k."""
    n = len(p)
    idx = np.empty((n, k), dtype=np.int32)
    d2 = np.empty((n, k), dtype=np.float64)
    _check(lib().abx_knn(p._h, int(k), _ptr(idx), _ptr(d2)), "abx_knn")
    return idx, d2


def spai_local_inverse_rows(op: Operator, k: int = 32):
    """Rows of the k-NN local block inverses (Schwarz block solves)."""
    n = op.shape[0]
    cols = np.empty((n, k), dtype=np.int32)
    vals = np.empty((n, k), dtype=np.float64)
    _check(lib().abx_spai_local_inverse_rows(op._h, int(k), _ptr(cols), _ptr(vals)),
           "abx_spai_local_inverse_rows")
    return cols, vals


def spai_exact_rows(op: Operator, k: int = 32):
    """Exact least-squares approximate-inverse rows on the k-NN support."""
    n = op.shape[0]
    cols = np.empty((n, k), dtype=np.int32)
    vals = np.empty((n, k), dtype=np.float64)
    _check(lib().abx_spai_exact_rows(op._h, int(k), _ptr(cols), _ptr(vals)), "abx_spai_exact_rows")
    return cols, vals


class MLP:
    """The learned preconditioner's model (``abx_mlp``)."""

    def __init__(self, h, ctx, out_dim):
        self._h = h
        self.ctx = ctx
        self.out_dim = out_dim

    @classmethod
    def create(cls, in_dim, hidden=128, nhidden=3, out_dim=32, seed=0, ctx=None):
        ctx = ctx or default_context()
        h = C.c_void_p()
        _check(lib().abx_mlp_create(ctx._h, int(in_dim), int(hidden), int(nhidden), int(out_dim),
                                    C.c_uint64(seed), C.byref(h)), "abx_mlp_create")
        return cls(h, ctx, int(out_dim))

    @classmethod
    def load(cls, path, ctx=None):
        ctx = ctx or default_context()
        h = C.c_void_p()
        _check(lib().abx_mlp_load(ctx._h, str(path).encode(), C.byref(h)), "abx_mlp_load")
        with open(path, "rb") as f:
            head = np.frombuffer(f.read(8 + 4 + 4 * 17), dtype=np.uint8)
        nl = int(np.frombuffer(head[8:12].tobytes(), np.int32)[0])
        dims = np.frombuffer(head[12:12 + 4 * (nl + 1)].tobytes(), np.int32)
        return cls(h, ctx, int(dims[-1]))

    def __del__(self):
        try:
            if self._h and not closing():
                lib().abx_mlp_destroy(self._h)
        except Exception:
            pass

    @property
    def num_params(self):
        return int(lib().abx_mlp_num_params(self._h))

    def save(self, path):
        _check(lib().abx_mlp_save(self._h, str(path).encode()), "abx_mlp_save")

    def set_normalization(self, in_scale, out_scale, out_shift):
        sc = np.ascontiguousarray(out_scale, dtype=np.float32)
        sh = np.ascontiguousarray(out_shift, dtype=np.float32)
        _check(lib().abx_mlp_set_normalization(self._h, float(in_scale), _ptr(sc), _ptr(sh)),
               "abx_mlp_set_normalization")

    def set_output_transform(self, kind, c=1.0):
        _check(lib().abx_mlp_set_output_transform(self._h, int(kind), float(c)),
               "abx_mlp_set_output_transform")

    @property
    def params(self):
        out = np.empty(self.num_params, dtype=np.float32)
        _check(lib().abx_mlp_get_params(self._h, _ptr(out)), "abx_mlp_get_params")
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().abx_mlp_set_params(self._h, _ptr(p)), "abx_mlp_set_params")

    def set_loss(self, kind, dim=0, kernel=None, cutoff=0.0):
        """LOSS_MSE (targets) or LOSS_SPAI_RESIDUAL (mean |A_i m_i - e_0|^2 with
        A_i built from each row's features by ``kernel`` inside ``cutoff``)."""
        _check(lib().abx_mlp_set_loss(self._h, int(kind), int(dim),
                                      C.byref(kernel) if kernel is not None else None,
                                      float(cutoff)), "abx_mlp_set_loss")

    def gradients(self, x, y=None):
        x = np.ascontiguousarray(x, dtype=np.float32)
        if y is not None:
            y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.num_params, dtype=np.float32)
        loss = C.c_float()
        _check(lib().abx_mlp_gradients(self._h, _ptr(x), _ptr(y), x.shape[0], _ptr(g),
                                       C.byref(loss)), "abx_mlp_gradients")
        return loss.value, g

    def train_step(self, x, y, lr):
        loss = C.c_float()
        if isinstance(x, np.ndarray):
            x = np.ascontiguousarray(x, dtype=np.float32)
            if y is not None:
                y = np.ascontiguousarray(y, dtype=np.float32)
        _check(lib().abx_mlp_train_step(self._h, _ptr(x), _ptr(y), int(x.shape[0]), float(lr),
                                        C.byref(loss)), "abx_mlp_train_step")
        return loss.value

    def forward(self, x, precision=PREC_MIXED):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], self.out_dim), dtype=np.float32)
        _check(lib().abx_mlp_forward(self._h, _ptr(x), x.shape[0], _ptr(y), int(precision)),
               "abx_mlp_forward")
        return y


def spai_features(p: Particles, knn_idx, eps):
    knn_idx = np.ascontiguousarray(knn_idx, dtype=np.int32)
    n, k = knn_idx.shape
    out = np.empty((n, k * p.dim), dtype=np.float32)
    _check(lib().abx_spai_features(p._h, _ptr(knn_idx), int(k), float(eps), _ptr(out)),
           "abx_spai_features")
    return out


def learned_preconditioner(op: Operator, mlp: MLP, eps: float, k: int = 32,
                           precision: int = PREC_MIXED, exact_phi: float = 0.5) -> Preconditioner:
    """The MLP's sparse approximate inverse; rows next to a neighbour with
    kernel value > exact_phi are solved exactly (exact_phi >= 1: none)."""
    h = C.c_void_p()
    _check(lib().abx_precond_create_learned(op._h, mlp._h, float(eps), int(k), int(precision),
                                            float(exact_phi), C.byref(h)),
           "abx_precond_create_learned")
    return Preconditioner(h, op.rows.ctx, op.shape[0], keep=(op, mlp))


def spai_rows(pc: Preconditioner, k: int = 32):
    cols = np.empty((pc.n, k), dtype=np.int32)
    vals = np.empty((pc.n, k), dtype=np.float64)
    _check(lib().abx_precond_get_spai(pc._h, _ptr(cols), _ptr(vals)), "abx_precond_get_spai")
    return cols, vals


def gmres_with_fallback(A: Operator, b, M_learned: Preconditioner | None, A_fallback: Operator,
                        restart=100, learned_max_iters=300, max_iters=2000, tol=1e-8,
                        A_check: Operator | None = None):
    """Learned preconditioner first; restricted additive Schwarz if it fails."""
    n = A.shape[0]
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    it, res, fb = C.c_int(), C.c_double(), C.c_int()
    _check(lib().abx_gmres_solve_fallback(A._h, A_check._h if A_check else None,
                                          M_learned._h if M_learned else None, A_fallback._h,
                                          _ptr(b), _ptr(x), int(restart), int(learned_max_iters),
                                          int(max_iters), float(tol), C.byref(it), C.byref(res),
                                          C.byref(fb)), "abx_gmres_solve_fallback")
    return x, it.value, res.value, bool(fb.value)


def create_fmm_operator(p: Particles, kernel: Kernel, order: int = 3,
                        precision: int = PREC_FP64) -> Operator:
    """``create_fmm_operator<order>`` on the octree of ``p``."""
    h = C.c_void_p()
    _check(lib().abx_create_fmm_operator(p._h, C.byref(kernel), int(order), C.byref(h)),
           "abx_create_fmm_operator")
    return Operator(h, p, p).set_precision(precision)


def create_h2_operator(p: Particles, kernel: Kernel, order: int = 3, eta: float = 1.0,
                       precision: int = PREC_FP64) -> Operator:
    """``create_h2_operator`` on an octree particle set: the black-box H2
    operator with runtime Chebyshev order and admissibility parameter eta."""
    h = C.c_void_p()
    _check(lib().abx_create_h2_operator(p._h, C.byref(kernel), int(order), float(eta),
                                        C.byref(h)), "abx_create_h2_operator")
    return Operator(h, p, p).set_precision(precision)


def fmm_set_wait_limit(op: Operator, seconds: float = 1.0, drop_one_arrive: bool = False):
    """Limit of the tensor-core M2L's device-side waits (``abx_fmm_set_wait_limit``);
    drop_one_arrive is the tests' fault injection (a barrier nothing arrives
    on), after which the matvec raises ABXError with status ABX_ERR_TIMEOUT."""
    _check(lib().abx_fmm_set_wait_limit(op._h, float(seconds), 1 if drop_one_arrive else 0),
           "abx_fmm_set_wait_limit")


def fmm_stats(op: Operator):
    a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
    t = C.c_double()
    _check(lib().abx_fmm_stats(op._h, C.byref(a), C.byref(b), C.byref(c), C.byref(t)), "fmm_stats")
    return {"m2l_pairs": a.value, "matrices": b.value, "leaves": c.value, "plan_s": t.value}


def fp32_peak_tflops(ctx: Context | None = None, packed: bool = True, iters: int = 4096) -> float:
    """Measured FP32 FMA throughput of the context's GPU in TFLOP/s
    (``abx_probe_fp32_peak``): the compute roofline's denominator."""
    ctx = ctx or default_context()
    out = C.c_double()
    _check(lib().abx_probe_fp32_peak(ctx._h, 1 if packed else 0, iters, C.byref(out)),
           "abx_probe_fp32_peak")
    return float(out.value)
