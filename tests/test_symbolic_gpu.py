"""The reference's Level-3 symbolic sums (src/Symbolic.h) through
include/aboria_gb/symbolic.cuh, in a program built by nvcc
(tests/cpp/symbolic_test.cu).

* CPU: the program compiles and links against the library.
* GPU: the known answers of the reference's tests/symbolic.h
  helper_neighbours (AccumulateWithinDistance sums in the 2- and inf-norm,
  univariate if_else and arithmetic assignments to positions and variables,
  eval of a sum over i of sums over j, scalar and vector, in a periodic
  domain), and
  on 20,000 random particles the neighbour count sum(j, norm(dx) < r, 1), the
  linear-spring sum of tests/speed_test.h:756-836 (the self pair taken out
  with if_else) and a dense sum(j, true, ...) against an FP64 brute force.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from aboria_gb300 import _lib
import workloads

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "symbolic_test.cu"


def _build(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    _lib.load_library()
    libdir = _lib.LIBPATH.parent
    exe = tmp_path / "symbolic_test"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "include"), str(SRC), "-L", str(libdir), "-labx",
                    "-Xlinker", f"-rpath={libdir}", "-o", str(exe)], check=True)
    return exe


def test_symbolic_program_builds(tmp_path):
    assert _build(tmp_path).exists()


@pytest.mark.gpu
def test_reference_symbolic_known_answers(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "kat"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "kat ok", r.stdout


@pytest.mark.gpu
def test_symbolic_sums_vs_brute_force(tmp_path):
    exe = _build(tmp_path)
    n, rad = 20000, 0.05
    pos = workloads.uniform(n, 3, seed=230)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n], np.int64).tofile(f)
        np.array([rad], np.float64).tofile(f)
        pos.tofile(f)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(exe), "run", str(inp), str(out)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    ids = np.fromfile(out / "ids.bin", np.int64)
    P = np.fromfile(out / "pos.bin", np.float64).reshape(n, 3)
    assert np.array_equal(P, pos[ids])
    count = np.fromfile(out / "count.bin", np.int32)
    spring = np.fromfile(out / "spring.bin", np.float64).reshape(n, 3)
    dense = np.fromfile(out / "dense.bin", np.float64)
    ref_count = np.zeros(n, np.int64)
    ref_spring = np.zeros((n, 3))
    ref_dense = np.zeros(n)
    for i0 in range(0, n, 1000):
        dx = P[None, :, :] - P[i0:i0 + 1000, None, :]        # x_j - x_i
        d = np.sqrt(((dx[..., 0] ** 2) + dx[..., 1] ** 2) + dx[..., 2] ** 2)
        near = d < rad
        ref_count[i0:i0 + 1000] = near.sum(1)
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(near & (d > 0), (rad - d) / d, 0.0)
        ref_spring[i0:i0 + 1000] = (w[..., None] * dx).sum(1)
        ref_dense[i0:i0 + 1000] = (1.0 / (1.0 + d * d)).sum(1)
    assert np.array_equal(count, ref_count)
    assert ref_count.min() >= 1 and ref_count.mean() > 5
    err = np.linalg.norm(spring - ref_spring) / np.linalg.norm(ref_spring)
    assert err < 1e-12, err
    assert np.max(np.abs(dense - ref_dense) / ref_dense) < 1e-12
