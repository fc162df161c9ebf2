"""ctypes loader for libabx.so (the CUDA library built from ``csrc/``).

The signatures are parsed from ``include/abx.h`` so the Python binding and the
C header cannot drift apart.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
HEADER = ROOT / "include" / "abx.h"
LIBPATH = PKG / "_build" / "libabx.so"


class ABXError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


_TYPES = {
    "void": None,
    "int": C.c_int,
    "double": C.c_double,
    "int64_t": C.c_int64,
    "uint64_t": C.c_uint64,
    "float": C.c_float,
    "uint32_t": C.c_uint32,
    "const char *": C.c_char_p,
}


def _ctype(t: str):
    t = " ".join(t.replace("*", " * ").split()).replace(" *", " *")
    if t.endswith("*"):
        base = t[:-1].strip()
        if base in ("const char", "char"):
            return C.c_char_p
        return C.c_void_p
    t = t.replace("const ", "")
    if t not in _TYPES:
        raise ValueError(f"unmapped C type {t!r}")
    return _TYPES[t]


def parse_header(path: Path = HEADER):
    """Return {name: (restype, [argtypes])} for every ABX_API declaration."""
    text = re.sub(r"/\*.*?\*/", "", path.read_text(), flags=re.S)
    decls = {}
    for m in re.finditer(r"ABX_API\s+([\w\s\*]+?)\s*\b(abx_\w+)\s*\(([^)]*)\)\s*;", text, re.S):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        ret = ret.strip()
        argtypes = []
        args = " ".join(args.split())
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                am = re.match(r"(.*?)(\w+)$", a)
                typ = am.group(1).strip() if am and am.group(1).strip() else a
                argtypes.append(_ctype(typ))
        decls[name] = (_ctype(ret) if ret != "void" else None, argtypes)
    return decls


_lib = None
_closing = False


def _mark_closing():
    global _closing
    _closing = True


def closing() -> bool:
    """True once the interpreter is shutting down: handle finalizers must not
    call into the library then (its CUDA runtime may already be torn down)."""
    import sys
    return _closing or sys.is_finalizing()


def load_library(path: Path | None = None):
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIBPATH
    if not p.exists():
        raise ABXError(-1, f"CUDA library {p} is not built; run __graft_entry__.build()")
    lib_ = C.CDLL(str(p))
    for name, (res, args) in parse_header().items():
        fn = getattr(lib_, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib_
    import atexit
    atexit.register(_mark_closing)
    return _lib


def lib():
    return load_library()
