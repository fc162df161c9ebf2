"""The C++ mirror of Aboria's API (include/aboria_gb/Aboria.h) compiled into a
program the way a reference user compiles against Aboria.

CPU: the header compiles with g++ and links against libabx.so, and a failing
call behaves like the reference's CHECK (message, then SIGTRAP) or, with
ABORIA_GB_THROW, throws std::runtime_error.
GPU: tests/cpp/api_test.cu built by nvcc (which adds the user-functor
operator) runs the neighbours/operators/RBF/FMM patterns of the reference's
tests; its outputs are compared with the oracle: storage order and neighbour
sets bit-exact, K*b to 1e-12, the functor operator against the built-in
kernel to 1e-12, the Schwarz-preconditioned GMRES residual, FMM to 1e-10.
"""
import json
import os
import shutil
import signal
import subprocess
from pathlib import Path

import numpy as np
import pytest

from aboria_gb300 import _lib
import oracle
import workloads

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "api_test.cu"
LIBDIR = _lib.LIBPATH.parent


def _gxx(tmp_path, extra=()):
    _lib.load_library()  # builds the library when it is missing
    exe = tmp_path / "api_test"
    cmd = ["g++", "-x", "c++", "-std=c++17", "-O1", "-Wall", "-Werror", *extra,
           "-I", str(ROOT / "include"), str(SRC), "-L", str(LIBDIR), "-labx",
           f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_header_compiles_and_failure_raises_sigtrap(tmp_path):
    exe = _gxx(tmp_path)
    r = subprocess.run([str(exe), "trap"], capture_output=True, text=True, timeout=120)
    assert r.returncode == -signal.SIGTRAP, (r.returncode, r.stderr)
    assert "CHECK failed" in r.stderr


def test_failure_throws_with_abori_gb_throw(tmp_path):
    exe = _gxx(tmp_path, ["-DABORIA_GB_THROW"])
    r = subprocess.run([str(exe), "throw"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("caught: ")


@pytest.mark.gpu
def test_cpp_api_parity(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    _lib.load_library()
    exe = tmp_path / "api_test_cu"
    subprocess.run([nvcc, "-std=c++17", "-O2", "--extended-lambda",
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "include"), str(SRC), "-L", str(LIBDIR), "-labx",
                    "-Xlinker", f"-rpath={LIBDIR}", "-o", str(exe)], check=True)
    n, nq, r, rw = 20000, 300, 0.08, 0.1
    pos = workloads.uniform(n, 3, seed=210)
    b = np.random.default_rng(211).standard_normal(n)
    q = workloads.uniform(nq, 3, seed=212)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, nq], np.int64).tofile(f)
        np.array([r, rw], np.float64).tofile(f)
        pos.tofile(f)
        b.tofile(f)
        q.tofile(f)
    out = tmp_path / "out"
    out.mkdir()
    res = subprocess.run([str(exe), "run", str(inp), str(out)], capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr

    cl = oracle.celllist_build(pos, [0, 0, 0], [1, 1, 1], [False] * 3, 10.0)
    ids = np.fromfile(out / "ids.bin", np.int64)
    assert np.array_equal(ids, cl.perm)

    counts = np.fromfile(out / "counts.bin", np.int32)
    lists = np.fromfile(out / "lists.bin", np.int32)
    rowptr, cols, _ = oracle.radius_lists(cl, q, r)
    assert np.array_equal(counts, np.diff(rowptr))
    off = np.concatenate([[0], np.cumsum(counts)])
    for k in range(nq):
        assert np.array_equal(np.sort(lists[off[k]:off[k + 1]]),
                              np.sort(cols[rowptr[k]:rowptr[k + 1]]))

    edit = np.fromfile(out / "edit.bin", np.float64)
    assert edit[0] == n + 1 and edit[1] == 1
    assert np.array_equal(edit[2:5], [0.123, 0.456, 0.789])
    assert edit[5] == n and edit[6] == 1 and edit[7] == 1

    bs = b[cl.perm]
    ref = oracle.sparse_matvec(cl, cl.pos, r, 1, [1.0 / (r / 2) ** 2], bs)
    kb = np.fromfile(out / "kb.bin", np.float64)
    assert np.max(np.abs(kb - ref)) <= 1e-12 * np.max(np.abs(ref))
    kf = np.fromfile(out / "kf.bin", np.float64)
    assert np.max(np.abs(kf - ref)) <= 1e-12 * np.max(np.abs(ref))
    # the closure on a periodic set (dx of the accepted image) against the
    # built-in kernel
    kbp = np.fromfile(out / "kbp.bin", np.float64)
    kfp = np.fromfile(out / "kfp.bin", np.float64)
    assert np.max(np.abs(kfp - kbp)) <= 1e-12 * np.max(np.abs(kbp))
    # the variable-radius operator against a brute force (non-periodic)
    kv = np.fromfile(out / "kv.bin", np.float64)
    rad = np.fromfile(out / "kv_radius.bin", np.float64)
    vid = np.fromfile(out / "kv_ids.bin", np.int64)
    P, bv = pos[vid], b[vid]
    want = np.empty(n)
    for i in range(n):
        dx = P - P[i]
        d2 = (dx[:, 0] * dx[:, 0] + dx[:, 1] * dx[:, 1]) + dx[:, 2] * dx[:, 2]
        m = ~(d2 > rad[i] * rad[i])
        want[i] = np.sum(np.exp(-d2[m] / (r / 2) ** 2) * bv[m])
    assert np.max(np.abs(kv - want)) <= 1e-12 * np.max(np.abs(want))
    assert len(np.unique(np.round(rad, 6))) > 100  # the radius does vary
    # the reference's block operator known answer (tests/operators.h:969-1090)
    bk = np.fromfile(out / "block_kat.bin", np.float64)
    want_block = json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())[
        "block_operator"]["answer"]
    assert np.all(np.abs(bk[:4] - want_block) <= np.finfo(float).eps), bk
    assert bk[4] == 4 and bk[5] == 4

    # the reference's sparse and block operator known answers, with the
    # user-functor path (tests/operators.h:810-963)
    kat = json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())["sparse_operator"]
    got = np.fromfile(out / "kat.bin", np.float64)
    assert np.array_equal(got[:3], kat["answer"])
    # the block answer: the entries the reference asserts, then the whole
    # vector against the product of the 6 x 3 block matrix its kernel defines
    assert np.array_equal(got[3:6], kat["block_answer_asserted"])
    C2 = np.array([[3, 3, 0], [-1, -1, 0], [3, 3, 3], [-1, -1, -1], [0, 3, 3], [0, -1, -1]], float)
    assert np.array_equal(got[3:9], C2 @ np.array([1.0, 2.0, 3.0]))
    assert got[9] == kat["nonzeros"] and got[10] == kat["block_nonzeros"]

    it, err, true_res = np.fromfile(out / "solve.bin", np.float64)
    assert err <= 1e-10 and true_res <= 1.0001e-10 and it < 500

    tree_ids = np.fromfile(out / "tree_ids.bin", np.int64)
    fmm = np.fromfile(out / "fmm.bin", np.float64)
    ref_f = oracle.fmm(pos[tree_ids], [0, 0, 0], [1, 1, 1], 64, 3, 5, [0.01], b[tree_ids])
    assert np.linalg.norm(fmm - ref_f) / np.linalg.norm(ref_f) < 1e-10
