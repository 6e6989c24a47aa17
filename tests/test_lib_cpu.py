"""CPU-side checks of the C ABI library: it loads without a GPU, exports
every function include/bilu_isai.h declares, and answers the host-only
queries (status strings, version, workspace sizes)."""
import ctypes
import os
import subprocess

import pytest

from isai_kernel_gb300 import _lib


def test_header_parses():
    decl = _lib.declarations()
    names = [d[0] for d in decl]
    assert len(names) == len(set(names)) and len(names) >= 45
    for must in ("bilu_bsrilu0", "bilu_isai_compute", "bilu_bcsr_spmv", "bilu_sptrsv",
                 "bilu_ctx_solve", "bilu_csr_to_bsr_fill", "bilu_map_bcsc2bcsr"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIBPATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for name, _, _ in _lib.declarations():
        assert name in exported, name
        assert getattr(L, name) is not None


def test_library_leaves_no_internal_symbol_undefined():
    """Every function of the library's own namespace is defined inside it
    (an undefined one only fails at load time on the GPU host)."""
    out = subprocess.run(["nm", "-D", "--undefined-only", _lib.LIBPATH], capture_output=True,
                         text=True, check=True).stdout
    missing = [ln.split()[-1] for ln in out.splitlines() if "_ZN4bilu" in ln]
    assert not missing, missing


def test_nested_mode_argument_checks():
    L = _lib.lib()
    assert L.bilu_ctx_set_inner(None, 8) == -1
    assert L.bilu_ctx_inner_steps(None, None) == -1
    h = ctypes.c_void_p()
    assert L.bilu_ctx_create(ctypes.byref(h), None) == 0
    assert L.bilu_ctx_set_inner(h, 0) == -1 and L.bilu_ctx_set_inner(h, 33) == -1
    assert L.bilu_ctx_set_inner(h, 8) == 0
    steps = ctypes.c_longlong(-1)
    assert L.bilu_ctx_inner_steps(h, ctypes.byref(steps)) == 0 and steps.value == 0
    # a solve before any setup is refused without touching a GPU
    assert L.bilu_ctx_solve(h, _lib.BILU_NESTED, ctypes.c_void_p(8), ctypes.c_void_p(16), 30,
                            ctypes.c_double(1e-10), 10, None, None, None) == -1
    assert L.bilu_ctx_destroy(h) == 0


def test_host_queries():
    L = _lib.lib()
    assert L.bilu_version() >= 10000
    assert L.bilu_status_string(-4) == b"sync-free wait timed out"
    assert L.bilu_status_string(0) == b"ok"
    assert L.bilu_bsrilu0_ws_bytes(1000, 5000) > 4000
    # level analysis scratch grows with the dependency count
    assert L.bilu_sptrsv_analysis_ws_bytes(1000, 9000) > L.bilu_sptrsv_analysis_ws_bytes(1000, 5000)
    assert L.bilu_sptrsv_ws_bytes(1000, 5000) >= L.bilu_sptrsv_solve_ws_bytes(1000)
    assert L.bilu_isai_pattern_ws_bytes(100, 500) > 0
    assert L.bilu_sptrsv_transpose_ws_bytes(10, 30, 4) > 30 * 16 * 8


def test_argument_errors_without_gpu():
    """Bad arguments are rejected before any CUDA call."""
    L = _lib.lib()
    assert L.bilu_bcsr_spmv(-1, 4, None, None, None, None, None, None) == -1
    assert L.bilu_bcsr_spmv(10, 6, ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8),
                            ctypes.c_void_p(8), ctypes.c_void_p(8), None) == -8
    assert L.bilu_bsrilu0(-2, 0, 4, None, None, None, None, None, 0, None) == -1
    assert L.bilu_isai_apply(10, 4, 7, None, None, None, None, None, None, None, None, None,
                             None) == -1
    lay = ctypes.c_int(7)
    assert L.bilu_spmv_layout(-1, 4, None, None, ctypes.byref(lay)) == -1
    assert L.bilu_spmv_layout(10, 4, ctypes.c_void_p(8), None, None) == -1
    assert L.bilu_spmv_layout(10, 6, ctypes.c_void_p(8), None, ctypes.byref(lay)) == -8
    assert lay.value == 7  # untouched on error
    assert L.bilu_debug_spmv_layout_set(10, 4, ctypes.c_void_p(8), 4) == -1  # only 0 .. 3
    assert L.bilu_debug_spmv_layout_set(10, 4, None, 1) == -1
    assert L.bilu_debug_spmv_layout_set(10, 6, ctypes.c_void_p(8), 1) == -8


def test_build_is_in_tree():
    assert os.path.dirname(_lib.LIBPATH).endswith("isai_kernel_gb300")
