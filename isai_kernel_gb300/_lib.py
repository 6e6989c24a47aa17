"""ctypes binding of libbilu_isai.so.

Argument and return types are read from include/bilu_isai.h, so the Python
side always matches the C ABI.  Loading fails loudly when the library has not
been built: there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "bilu_isai.h")
LIBPATH = os.path.join(HERE, "libbilu_isai.so")

_CT = {
    "int": ctypes.c_int,
    "long long": ctypes.c_longlong,
    "unsigned long long": ctypes.c_ulonglong,
    "size_t": ctypes.c_size_t,
    "double": ctypes.c_double,
    "void": None,
    "const char*": ctypes.c_char_p,
}

STATUS = {
    0: "BILU_OK",
    -1: "BILU_ERR_ARG",
    -2: "BILU_ERR_PATTERN",
    -3: "BILU_ERR_ZERO_PIVOT",
    -4: "BILU_ERR_TIMEOUT",
    -5: "BILU_ERR_CUDA",
    -6: "BILU_ERR_NOT_CONVERGED",
    -7: "BILU_ERR_WORKSPACE",
    -8: "BILU_ERR_UNSUPPORTED",
    -9: "BILU_ERR_IO",
}
BILU_FP64, BILU_FP32, BILU_ILU, BILU_FP32_INNER, BILU_ILU_FP32, BILU_NESTED = 0, 1, 2, 3, 4, 5


def _ctype(t: str):
    t = " ".join(t.replace("*", " * ").split()).replace(" *", "*")
    if t in _CT:
        return _CT[t]
    if t.endswith("*"):
        return ctypes.c_void_p
    if t == "bilu_stream_t":
        return ctypes.c_void_p
    raise ValueError(f"unmapped C type {t!r}")


def declarations(header: str = HEADER):
    """(name, restype, [argtypes]) for every function declared in the header."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = []
    for m in re.finditer(r"([A-Za-z_][\w \*]*?)\b(bilu_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("typedef"):
            continue
        argtypes = []
        if args and args != "void":
            for a in args.split(","):
                a = " ".join(a.split())
                am = re.match(r"(.*?)([A-Za-z_]\w*)$", a)
                argtypes.append(_ctype(am.group(1).strip()))
        out.append((name, _ctype(ret), argtypes))
    return out


_LIB = None


class BiluError(RuntimeError):
    def __init__(self, func: str, status: int):
        self.status = status
        self.func = func
        msg = _LIB.bilu_status_string(status).decode() if _LIB is not None else ""
        self.cuda_error = _LIB.bilu_last_cuda_error() if _LIB is not None else 0
        if status == -5:  # BILU_ERR_CUDA
            msg += f" (cudaError_t {self.cuda_error})"
        super().__init__(f"{func} returned {STATUS.get(status, status)}: {msg}")


def lib():
    """Load libbilu_isai.so (built by isai_kernel_gb300.build)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(
                f"{LIBPATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'` (nvcc, sm_103a)")
        L = ctypes.CDLL(LIBPATH)
        for name, res, args in declarations():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def check(func: str, status: int, ok=(0,)) -> int:
    if status not in ok:
        raise BiluError(func, status)
    return status


def call(name: str, *args, ok=(0,)):
    """Call an int-returning entry point and raise BiluError on failure."""
    return check(name, getattr(lib(), name)(*args), ok)
