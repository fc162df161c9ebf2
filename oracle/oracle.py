"""Python handle on the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/liboracle.so`` (built from ``aboria_oracle.cpp`` by
``build_oracle.sh``), a C++ restatement of the reference algorithms.  Only the
test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, always as the checker or the timed CPU baseline, never as
part of the product path.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def build() -> Path:
    subprocess.run(["sh", str(HERE / "build_oracle.sh")], check=True, capture_output=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "aboria_oracle.cpp").stat().st_mtime:
            build()
        _lib = C.CDLL(str(LIB))
        _lib.orc_grid.restype = C.c_uint32
        _lib.orc_collapse.restype = C.c_uint32
        _lib.orc_point_to_bucket.restype = C.c_int
        _lib.orc_celllist_build.restype = C.c_int64
        _lib.orc_octree_build.restype = C.c_int64
        _lib.orc_num_threads.restype = C.c_int
        for name in ("orc_radius_count", "orc_radius_lists", "orc_sparse_matvec", "orc_schwarz_apply",
                     "orc_fmm", "orc_direct_sum",
                     "orc_dense_matvec", "orc_brute_counts", "orc_set_num_threads",
                     "orc_reassemble"):
            getattr(_lib, name).restype = None
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_num_threads(n: int):
    lib().orc_set_num_threads(C.c_int(n))


@dataclass
class CellList:
    dim: int
    lo: np.ndarray
    hi: np.ndarray
    periodic: np.ndarray
    size: np.ndarray
    side: np.ndarray
    pos: np.ndarray        # sorted positions (n_alive, dim)
    perm: np.ndarray       # original index of each sorted particle
    keys: np.ndarray
    begin: np.ndarray
    end: np.ndarray
    pos_enforced: np.ndarray  # input positions after the periodic wrap

    @property
    def n(self):
        return self.pos.shape[0]


def grid(dim, lo, hi, periodic, n_leaf, n_alive):
    size = np.zeros(3, np.uint32)
    side = np.zeros(3, np.float64)
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    per = np.ascontiguousarray([1 if p else 0 for p in periodic], np.int32)
    nc = lib().orc_grid(C.c_int(dim), _p(lo), _p(hi), _p(per), C.c_double(n_leaf),
                        C.c_int64(n_alive), _p(size), _p(side))
    return size[:dim], side[:dim], int(nc)


def collapse(size, v):
    size = np.ascontiguousarray(size, np.uint32)
    v = np.ascontiguousarray(v, np.int32)
    return int(lib().orc_collapse(C.c_int(len(size)), _p(size), _p(v)))


def reassemble(size, index):
    size = np.ascontiguousarray(size, np.uint32)
    v = np.zeros(len(size), np.int32)
    lib().orc_reassemble(C.c_int(len(size)), _p(size), C.c_uint32(index), _p(v))
    return v


def point_to_bucket(size, lo, side, x):
    size = np.ascontiguousarray(size, np.uint32)
    lo = np.ascontiguousarray(lo, np.float64)
    side = np.ascontiguousarray(side, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    v = np.zeros(len(size), np.int32)
    idx = lib().orc_point_to_bucket(C.c_int(len(size)), _p(size), _p(lo), _p(side), _p(x), _p(v))
    return int(idx), v


def celllist_build(pos, lo, hi, periodic, n_leaf=10.0, stable=True, prev_grid_n=0) -> CellList:
    """Domain enforcement, grid, stable sort and bucket ranges.  prev_grid_n:
    the alive count the existing grid was computed with (0: none); the grid
    is kept while the new alive count stays within a factor 2 of it."""
    pos = np.array(pos, dtype=np.float64, order="C", copy=True)
    n, dim = pos.shape
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    per = np.ascontiguousarray([1 if p else 0 for p in periodic], np.int32)
    _, _, nc_cap = grid(dim, lo, hi, periodic, n_leaf, max(n, prev_grid_n))
    # the grid of the alive count can only be smaller or equal in most cases;
    # retry with a larger capacity if not.
    cap = max(nc_cap, 1) * 8 + 64
    while True:
        pos_io = pos.copy()
        out_pos = np.zeros((n, dim))
        perm = np.zeros(n, np.int64)
        keys = np.zeros(n, np.uint32)
        bb = np.zeros(cap, np.uint32)
        be = np.zeros(cap, np.uint32)
        size = np.zeros(3, np.uint32)
        side = np.zeros(3, np.float64)
        gn = np.zeros(1, np.int64)
        na = lib().orc_celllist_build(C.c_int(dim), C.c_int64(n), _p(pos_io), _p(lo), _p(hi),
                                      _p(per), C.c_double(n_leaf), C.c_int(1 if stable else 0),
                                      _p(out_pos), _p(perm), _p(keys), _p(bb), _p(be),
                                      C.c_uint32(cap), _p(size), _p(side),
                                      C.c_int64(prev_grid_n), _p(gn))
        if na >= 0:
            break
        cap *= 8
    nc = int(np.prod(size[:dim].astype(np.int64)))
    return CellList(dim, lo, hi, per, size[:dim].copy(), side[:dim].copy(), out_pos[:na].copy(),
                    perm[:na].copy(), keys[:na].copy(), bb[:nc].copy(), be[:nc].copy(), pos_io)


def _grid_args(cl: CellList):
    size = np.ones(3, np.uint32)
    side = np.ones(3, np.float64)
    size[:cl.dim] = cl.size
    side[:cl.dim] = cl.side
    return size, side


def radius_count(cl: CellList, q, r, lnorm=2):
    """Neighbour counts; lnorm 2 / 1 / -1 = euclidean_search / manhatten_search
    / chebyshev_search (src/Search.h:797-845)."""
    q = np.ascontiguousarray(q, np.float64).reshape(-1, cl.dim)
    size, side = _grid_args(cl)
    out = np.zeros(q.shape[0], np.int32)
    lib().orc_radius_count(C.c_int(cl.dim), _p(size), _p(cl.lo), _p(cl.hi), _p(cl.periodic),
                           _p(side), C.c_int64(cl.n), _p(np.ascontiguousarray(cl.pos)),
                           _p(cl.begin), _p(cl.end), C.c_int64(q.shape[0]), _p(q), C.c_double(r),
                           C.c_int(lnorm), _p(out))
    return out


def radius_lists(cl: CellList, q, r, with_dx=False, lnorm=2):
    """Neighbour lists in the reference's visiting order (CSR), norm as for
    radius_count."""
    q = np.ascontiguousarray(q, np.float64).reshape(-1, cl.dim)
    counts = radius_count(cl, q, r, lnorm)
    rowptr = np.zeros(q.shape[0] + 1, np.int64)
    np.cumsum(counts, out=rowptr[1:])
    nnz = int(rowptr[-1])
    cols = np.zeros(max(nnz, 1), np.int64)
    dx = np.zeros((max(nnz, 1), cl.dim)) if with_dx else None
    size, side = _grid_args(cl)
    lib().orc_radius_lists(C.c_int(cl.dim), _p(size), _p(cl.lo), _p(cl.hi), _p(cl.periodic),
                           _p(side), C.c_int64(cl.n), _p(np.ascontiguousarray(cl.pos)),
                           _p(cl.begin), _p(cl.end), C.c_int64(q.shape[0]), _p(q), C.c_double(r),
                           C.c_int(lnorm), _p(rowptr), _p(cols), _p(dx))
    return rowptr, cols[:nnz], (dx[:nnz] if with_dx else None)


def sparse_matvec(cl: CellList, row_pos, r, kind, params, b, row_s=None, col_s=None):
    row_pos = np.ascontiguousarray(row_pos, np.float64).reshape(-1, cl.dim)
    b = np.ascontiguousarray(b, np.float64)
    prm = np.zeros(4)
    prm[:len(params)] = params
    c = np.zeros(row_pos.shape[0])
    size, side = _grid_args(cl)
    rs = None if row_s is None else np.ascontiguousarray(row_s, np.float64)
    cs = None if col_s is None else np.ascontiguousarray(col_s, np.float64)
    lib().orc_sparse_matvec(C.c_int(cl.dim), _p(size), _p(cl.lo), _p(cl.hi), _p(cl.periodic),
                            _p(side), C.c_int64(cl.n), _p(np.ascontiguousarray(cl.pos)),
                            _p(cl.begin), _p(cl.end), C.c_int64(row_pos.shape[0]), _p(row_pos),
                            C.c_double(r), C.c_int(kind), _p(prm), _p(rs), _p(cs), _p(b), _p(c))
    return c


def dense_matvec(row_pos, col_pos, kind, params, b, row_s=None, col_s=None):
    row_pos = np.ascontiguousarray(row_pos, np.float64)
    col_pos = np.ascontiguousarray(col_pos, np.float64)
    dim = row_pos.shape[1]
    b = np.ascontiguousarray(b, np.float64)
    prm = np.zeros(4)
    prm[:len(params)] = params
    c = np.zeros(row_pos.shape[0])
    rs = None if row_s is None else np.ascontiguousarray(row_s, np.float64)
    cs = None if col_s is None else np.ascontiguousarray(col_s, np.float64)
    lib().orc_dense_matvec(C.c_int(dim), C.c_int64(row_pos.shape[0]), _p(row_pos),
                           C.c_int64(col_pos.shape[0]), _p(col_pos), C.c_int(kind), _p(prm),
                           _p(rs), _p(cs), _p(b), _p(c))
    return c


def brute_counts(pos, lo, hi, periodic: bool, r):
    pos = np.ascontiguousarray(pos, np.float64)
    n, dim = pos.shape
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    out = np.zeros(n, np.int32)
    lib().orc_brute_counts(C.c_int(dim), C.c_int64(n), _p(pos), _p(lo), _p(hi),
                           C.c_int(1 if periodic else 0), C.c_double(r), _p(out))
    return out


@dataclass
class Octree:
    perm: np.ndarray
    tags: np.ndarray
    leaf_level: np.ndarray
    leaf_tag: np.ndarray
    leaf_begin: np.ndarray
    leaf_end: np.ndarray


def octree_build(pos, lo, hi, n_leaf):
    """HyperOctree on already domain-enforced positions (no deletion)."""
    pos = np.ascontiguousarray(pos, np.float64)
    n, dim = pos.shape
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    perm = np.zeros(n, np.int64)
    tags = np.zeros(n, np.int32)
    cap = max(16, n) * 2
    lv, lt, lb, le = (np.zeros(cap, np.int32) for _ in range(4))
    nl = lib().orc_octree_build(C.c_int(dim), C.c_int64(n), _p(pos), _p(lo), _p(hi),
                                C.c_double(n_leaf), _p(perm), _p(tags), _p(lv), _p(lt), _p(lb),
                                _p(le), C.c_int64(cap))
    assert nl >= 0
    return Octree(perm, tags, lv[:nl].copy(), lt[:nl].copy(), lb[:nl].copy(), le[:nl].copy())


def schwarz_apply(pos, lo, hi, periodic, tree: Octree, radius, kind, params, b):
    """Restricted additive Schwarz on octree leaves (tree-ordered positions)."""
    pos = np.ascontiguousarray(pos, np.float64)
    n, dim = pos.shape
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    per = np.ascontiguousarray([1 if p else 0 for p in periodic], np.int32)
    prm = np.zeros(4)
    prm[:len(params)] = params
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(n)
    lib().orc_schwarz_apply(C.c_int(dim), C.c_int64(n), _p(pos), _p(lo), _p(hi), _p(per),
                            C.c_int64(len(tree.leaf_level)), _p(tree.leaf_level),
                            _p(tree.leaf_tag), _p(tree.leaf_begin), _p(tree.leaf_end),
                            C.c_double(radius), C.c_int(kind), _p(prm), _p(b), _p(x))
    return x


def fmm(pos, lo, hi, n_leaf, order, kind, params, b):
    """Black-box Chebyshev FMM restatement; output in input order."""
    pos = np.ascontiguousarray(pos, np.float64)
    npts, dim = pos.shape
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    prm = np.zeros(4)
    prm[:len(params)] = params
    b = np.ascontiguousarray(b, np.float64)
    c = np.zeros(npts)
    lib().orc_fmm(C.c_int(dim), C.c_int(order), C.c_int64(npts), _p(pos), _p(lo), _p(hi),
                  C.c_double(n_leaf), C.c_int(kind), _p(prm), _p(b), _p(c))
    return c


def direct_sum(pos, kind, params, b, targets, skip_self=False):
    """FP64 direct sum c_t = sum_j K(x_j - x_i) b_j, i = targets[t], j in input
    order; skip_self leaves out j == i."""
    pos = np.ascontiguousarray(pos, np.float64)
    npts, dim = pos.shape
    prm = np.zeros(4)
    prm[:len(params)] = params
    targets = np.ascontiguousarray(targets, np.int64)
    c = np.zeros(len(targets))
    lib().orc_direct_sum(C.c_int(dim), C.c_int64(npts), _p(pos), C.c_int(kind), _p(prm),
                         _p(np.ascontiguousarray(b, np.float64)), C.c_int64(len(targets)),
                         _p(targets), C.c_int(1 if skip_self else 0), _p(c))
    return c
