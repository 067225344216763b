"""ctypes binding of libgbla.so.

The argument and return types of every entry point are read from
``include/gbla.h`` itself, so the binding cannot drift from the C ABI.  The
library is loaded from the package directory; if it is missing the import
fails loudly (there is no fallback implementation).
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "gbla.h")
LIB_PATH = os.path.join(HERE, "libgbla.so")

_CTYPES = {
    "int": C.c_int,
    "unsigned int": C.c_uint,
    "int64_t": C.c_int64,
    "uint64_t": C.c_uint64,
    "size_t": C.c_size_t,
    "float": C.c_float,
    "double": C.c_double,
    "char": C.c_char,
    "gbla_status": C.c_int,
    "gbla_gemm_mode": C.c_int,
    "cudaStream_t": C.c_void_p,
    "void": None,
}

_DECL = re.compile(r"^\s*([A-Za-z_][\w\s\*]*?)\s*\b(gbla_\w+)\s*\(([^;]*?)\)\s*;", re.M | re.S)


def _ctype(tok: str):
    tok = " ".join(tok.replace("const", " ").split())
    if "*" in tok:
        base = tok.replace("*", "").strip()
        return C.c_char_p if base == "char" else C.c_void_p
    if tok not in _CTYPES:
        raise TypeError(f"unmapped C type {tok!r} in gbla.h")
    return _CTYPES[tok]


def parse_header(path: str = HEADER):
    """Return {name: (restype, [argtypes])} for every function in gbla.h."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    out = {}
    for ret, name, args in _DECL.findall(text):
        ret = ret.strip()
        if ret.startswith("typedef") or "(" in ret:
            continue
        argtypes = []
        args = " ".join(args.split())
        if args and args != "void":
            for a in args.split(","):
                a = a.strip()
                # drop the parameter name
                m = re.match(r"(.*?)([A-Za-z_]\w*)$", a)
                argtypes.append(_ctype(m.group(1) if m and m.group(1).strip() else a))
        out[name] = (_ctype(ret), argtypes)
    return out


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run gputils_gb300.build.build_lib() first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in parse_header().items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class GblaError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status != 0:
        name = lib().gbla_status_string(status).decode()
        raise GblaError(f"{what}: {name} (last CUDA error {lib().gbla_last_cuda_error()})")


def call(name: str, *args) -> None:
    """Call a gbla_* entry point that returns gbla_status; raise on failure."""
    check(getattr(lib(), name)(*args), name)
