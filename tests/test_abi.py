"""The C ABI library loads and exports exactly what include/abx.h declares.

Runs without a GPU: no compute call is made (only calls that fail cleanly on a
machine without a device).
"""
import ctypes as C
import subprocess

import pytest

from aboria_gb300 import _lib


def test_header_parses_and_library_exports_every_symbol():
    decls = _lib.parse_header()
    assert len(decls) >= 28
    lib = _lib.load_library()
    for name in decls:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIBPATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(decls) <= exported
    # nothing else leaks out of the library under the abx_ prefix
    assert {s for s in exported if s.startswith("abx_")} == set(decls)


def test_version_and_error_string():
    lib = _lib.load_library()
    assert lib.abx_version() >= 1
    assert isinstance(lib.abx_last_error(), bytes)


def test_null_arguments_are_rejected_without_touching_the_device():
    lib = _lib.load_library()
    assert lib.abx_context_create(0, None, None) == 1  # ABX_ERR_INVALID
    assert b"null" in lib.abx_last_error()
    assert lib.abx_particles_create(None, 3, None) == 1
    assert lib.abx_operator_matvec(None, None, None) == 1
    assert lib.abx_radius_count(None, 0, None, 0.1, None) == 1


def test_context_create_fails_cleanly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load_library()
    h = C.c_void_p()
    st = lib.abx_context_create(0, None, C.byref(h))
    assert st != 0
    assert len(lib.abx_last_error()) > 0
