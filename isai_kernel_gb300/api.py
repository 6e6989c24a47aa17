"""Host-side mirror of the reference's entry points on CUDA tensors.

Each function keeps the reference's name and argument meaning (gmfff/isai_kernel,
file:line in the docstring) and calls the matching C ABI entry point of
libbilu_isai.so.  Inputs are torch CUDA tensors (int32 indices, float64 /
float32 values); block size is a runtime argument.  Errors raise BiluError
where the reference calls exit(1).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import torch

from ._lib import (BILU_FP32, BILU_FP32_INNER, BILU_FP64, BILU_ILU, BILU_ILU_FP32, BILU_NESTED,
                   BiluError, call, lib)

_I32, _F64, _F32 = torch.int32, torch.float64, torch.float32


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _s(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ws(nbytes: int, dev):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=dev)


def _dev(*ts):
    for t in ts:
        if not t.is_cuda:
            raise ValueError("expected CUDA tensors")
    return ts[0].device


# Contiguous copies made for a call stay referenced until the next call
# built from them: arguments are evaluated before the launch, and a copy
# freed in between could hand its memory to the next argument's copy.  (Once
# the kernel is queued, the stream-ordered allocator makes the release safe.)
_held: list = []


def _hold(t, orig):
    if t.data_ptr() != orig.data_ptr():
        if len(_held) > 64:
            del _held[:32]
        _held.append(t)
    return t


def _ci(t):
    c = t.contiguous()
    if c.dtype != _I32:
        raise TypeError("index arrays must be int32")
    return _hold(c, t)


def _cf(t, dtype=_F64):
    c = t.contiguous()
    if c.dtype != dtype:
        raise TypeError(f"values must be {dtype}")
    return _hold(c, t)


# ------------------------------------------------------------ conversions
def csr_to_bsr5(n: int, bs: int, csrRowPtr, csrColInd, csrVal):
    """csr2bsr.h:14 csr_to_bsr5 -> (nb, bsrRowPtr, bsrColInd, bsrVal[nnzb,bs,bs])."""
    dev = _dev(csrRowPtr, csrColInd, csrVal)
    rp, ci, v = _ci(csrRowPtr), _ci(csrColInd), _cf(csrVal)
    nb = n // bs
    brow = torch.empty(nb + 1, dtype=_I32, device=dev)
    nnzb = ctypes.c_int(0)
    ws = _ws(lib().bilu_csr_to_bsr_ws_bytes(n, bs), dev)
    call("bilu_csr_to_bsr_rowptr", n, bs, _p(rp), _p(ci), _p(brow), ctypes.byref(nnzb), _p(ws),
         ws.numel(), _s())
    bcol = torch.empty(nnzb.value, dtype=_I32, device=dev)
    bval = torch.empty((nnzb.value, bs, bs), dtype=_F64, device=dev)
    call("bilu_csr_to_bsr_fill", n, bs, _p(rp), _p(ci), _p(v), _p(brow), _p(bcol), _p(bval),
         _s())
    return nb, brow, bcol, bval


def bsr2csr(mb: int, bs: int, bsrRowPtr, bsrColInd, bsrVal):
    """bsr2csr.h:19 bsr2csr_cusparse (row direction) -> (csrRowPtr, csrColInd, csrVal)."""
    dev = _dev(bsrRowPtr)
    nnzb = int(bsrColInd.numel())
    rp = torch.empty(mb * bs + 1, dtype=_I32, device=dev)
    ci = torch.empty(nnzb * bs * bs, dtype=_I32, device=dev)
    v = torch.empty(nnzb * bs * bs, dtype=_F64, device=dev)
    call("bilu_bsr_to_csr", mb, bs, _p(_ci(bsrRowPtr)), _p(_ci(bsrColInd)), _p(_cf(bsrVal)),
         _p(rp), _p(ci), _p(v), _s())
    return rp, ci, v


def build_bcsc_pattern_from_bsr_scalarILU(nb: int, Abrow, Abcol, for_lower: bool):
    """isai_bsr.h:246 -> (Mbrow, Mcol) BCSC pattern of M_L / M_U."""
    dev = _dev(Abrow, Abcol)
    ar, ac = _ci(Abrow), _ci(Abcol)
    mp = torch.empty(nb + 1, dtype=_I32, device=dev)
    nnz = ctypes.c_int(0)
    ws = _ws(lib().bilu_isai_pattern_ws_bytes(nb, int(ac.numel())), dev)
    call("bilu_isai_pattern_colptr", nb, _p(ar), _p(ac), int(for_lower), _p(mp),
         ctypes.byref(nnz), _p(ws), ws.numel(), _s())
    mi = torch.empty(nnz.value, dtype=_I32, device=dev)
    call("bilu_isai_pattern_fill", nb, _p(ar), _p(ac), int(for_lower), _p(mp), _p(mi), _p(ws),
         ws.numel(), _s())
    return mp, mi


def pattern_product(nb: int, Xrow, Xcol, Arow, Acol):
    """Symbolic block-pattern product pattern(X A) -> (rowptr, colind)
    (bilu_pattern_product_*; ISAI(k) patterns are pattern(A^k))."""
    dev = _dev(Xrow)
    cr = torch.empty(nb + 1, dtype=_I32, device=dev)
    nnz, bad = ctypes.c_int(0), ctypes.c_int(-1)
    ws = _ws(lib().bilu_pattern_product_ws_bytes(nb), dev)
    xr, xc, ar, ac = _ci(Xrow), _ci(Xcol), _ci(Arow), _ci(Acol)
    call("bilu_pattern_product_rowptr", nb, _p(xr), _p(xc), _p(ar), _p(ac), _p(cr),
         ctypes.byref(nnz), ctypes.byref(bad), _p(ws), ws.numel(), _s())
    cc = torch.empty(max(nnz.value, 1), dtype=_I32, device=dev)
    call("bilu_pattern_product_fill", nb, _p(xr), _p(xc), _p(ar), _p(ac), _p(cr), _p(cc), _p(ws),
         ws.numel(), _s())
    return cr, cc[: nnz.value]


def build_triangular_bcsr_pattern_from_A(nb: int, A_bsrRow, A_bsrCol, lower: bool):
    """bcsc2bcsr.h:11 -> (T_bsrRow, T_bsrCol)."""
    dev = _dev(A_bsrRow)
    ar, ac = _ci(A_bsrRow), _ci(A_bsrCol)
    tr = torch.empty(nb + 1, dtype=_I32, device=dev)
    nnz = ctypes.c_int(0)
    ws = _ws(lib().bilu_tri_pattern_ws_bytes(nb), dev)
    call("bilu_tri_pattern_rowptr", nb, _p(ar), _p(ac), int(lower), _p(tr), ctypes.byref(nnz),
         _p(ws), ws.numel(), _s())
    tc = torch.empty(nnz.value, dtype=_I32, device=dev)
    call("bilu_tri_pattern_fill", nb, _p(ar), _p(ac), int(lower), _p(tr), _p(tc), _s())
    return tr, tc


def build_map_bcsc2bcsr_host(nb: int, bcscColPtr, bcscRowInd, bcsrRowPtr, bcsrColInd):
    """bcsc2bcsr.h:32 -> map_bcsc2bcsr.  Raises BiluError (BILU_ERR_PATTERN,
    .bad = (row, col)) where the reference exits."""
    dev = _dev(bcscColPtr)
    m = torch.empty(int(bcscRowInd.numel()), dtype=_I32, device=dev)
    bad = (ctypes.c_int * 2)(-1, -1)
    ws = _ws(lib().bilu_map_ws_bytes(), dev)
    st = lib().bilu_map_bcsc2bcsr(nb, _p(_ci(bcscColPtr)), _p(_ci(bcscRowInd)),
                                  _p(_ci(bcsrRowPtr)), _p(_ci(bcsrColInd)), _p(m), bad, _p(ws),
                                  ws.numel(), _s())
    if st != 0:
        e = BiluError("bilu_map_bcsc2bcsr", st)
        e.bad = (bad[0], bad[1])
        raise e
    return m


def reorder_bcsc_val_to_bcsr(map_bcsc2bcsr, bcsc_val):
    """bcsc2bcsr.h:63 reorder_bcsc_val_to_bcsr_bs5 -> bcsr_val."""
    v = _cf(bcsc_val)
    bs = v.shape[-1]
    out = torch.empty_like(v)
    call("bilu_reorder_bcsc_to_bcsr", int(map_bcsc2bcsr.numel()), bs, _p(_ci(map_bcsc2bcsr)),
         _p(v), _p(out), _s())
    return out


def bcsc_to_bcsr(MB: int, NB: int, bs: int, colPtr, rowInd, val):
    """bcsc2bcsrAndSpMV.h:76 bcsc_to_bcsr (deterministic) -> (row_ptr, col_ind, val)."""
    dev = _dev(colPtr)
    nnzb = int(rowInd.numel())
    rp = torch.empty(MB + 1, dtype=_I32, device=dev)
    ci = torch.empty(nnzb, dtype=_I32, device=dev)
    v = torch.empty((nnzb, bs, bs), dtype=_F64, device=dev)
    ws = _ws(lib().bilu_bcsc_to_bcsr_ws_bytes(MB, nnzb), dev)
    call("bilu_bcsc_to_bcsr", MB, NB, bs, _p(_ci(colPtr)), _p(_ci(rowInd)),
         _p(None if val is None else _cf(val)), _p(rp), _p(ci), _p(v), _p(ws), ws.numel(), _s())
    return rp, ci, v


def bsr_transpose(mb: int, bs: int, row, col, val):
    """BCSC view of a BCSR matrix as BCSR of the transpose (blocks transposed)."""
    dev = _dev(row)
    nnzb = int(col.numel())
    tr = torch.empty(mb + 1, dtype=_I32, device=dev)
    tc = torch.empty(nnzb, dtype=_I32, device=dev)
    tv = torch.empty((nnzb, bs, bs), dtype=_F64, device=dev)
    ws = _ws(lib().bilu_bsr_transpose_ws_bytes(mb, nnzb), dev)
    call("bilu_bsr_transpose", mb, bs, _p(_ci(row)), _p(_ci(col)), _p(_cf(val)), _p(tr), _p(tc),
         _p(tv), _p(ws), ws.numel(), _s())
    return tr, tc, tv


# ------------------------------------------------------------ factorisation
def bsrilu02_inplace(nb: int, nnzb: int, bs: int, bsrRow, bsrCol, bsrVal,
                     schedule: int = -1) -> int:
    """bsrilu.h:20 bsrilu02_inplace: BILU(0) in place (schedule: -1 as the
    level analysis recommends, 0 level, 1 sync-free).  Returns the first
    zero-pivot block row or -1 (the reference prints it)."""
    dev = _dev(bsrVal)
    info = ctypes.c_int(-1)
    ws = _ws(lib().bilu_bsrilu0_ws_bytes(nb, nnzb), dev)
    call("bilu_bsrilu0_ex", nb, nnzb, bs, _p(_ci(bsrRow)), _p(_ci(bsrCol)), _p(bsrVal), schedule,
         ctypes.byref(info), _p(ws), ws.numel(), _s(), ok=(0, -3))
    return info.value


# ------------------------------------------------------------ ISAI setup
def build_Dinv(nb: int, bs: int, Abrow, Abcol, Abval, lower: bool):
    """isai_bsr.h:91 build_DinvL_from_BSR5_kernel_fix (lower) /
    isai_bsr.h:126 build_DinvU_from_BSR5_kernel_fix -> Dinv[nb, bs, bs]."""
    out = torch.empty((nb, bs, bs), dtype=_F64, device=_dev(Abval))
    call("bilu_build_dinv", nb, bs, _p(_ci(Abrow)), _p(_ci(Abcol)), _p(_cf(Abval)), int(lower),
         _p(out), _s())
    return out


def build_pairs(nb: int, Abrow, Abcol, Mbrow, Mcol, lower: bool = True):
    """isai_bsr.h:1378 count_pairs_lower_kernel_v2 + main.cu:684 scan +
    isai_bsr.h:1427 fill_pairs_lower_kernel_v2 (lower=False: the M_U list)
    -> (PairPtr, PairPLocal, PairSrc, Nmax)."""
    dev = _dev(Mbrow)
    mnnz = int(Mcol.numel())
    pp = torch.empty(mnnz + 1, dtype=_I32, device=dev)
    total, nmax = ctypes.c_int(0), ctypes.c_int(0)
    ws = _ws(lib().bilu_pairs_ws_bytes(mnnz), dev)
    ar, ac, mp, mi = _ci(Abrow), _ci(Abcol), _ci(Mbrow), _ci(Mcol)
    call("bilu_pairs_ptr", nb, _p(ar), _p(ac), _p(mp), _p(mi), int(lower), _p(pp),
         ctypes.byref(total), ctypes.byref(nmax), _p(ws), ws.numel(), _s())
    pl = torch.empty(total.value, dtype=_I32, device=dev)
    ps = torch.empty(total.value, dtype=_I32, device=dev)
    call("bilu_pairs_fill", nb, _p(ar), _p(ac), _p(mp), _p(mi), int(lower), _p(pp), _p(pl),
         _p(ps), _s())
    return pp, pl, ps, nmax.value


def isai_compute(nb: int, bs: int, Abval, Mbrow, Mcol, PairPtr, PairPLocal, PairSrc, Dinv,
                 lower: bool):
    """isai_bsr.h:288 (lower) / :161 (upper) ISAI column solves -> Mval[Mnnz, bs, bs]
    in BCSC order."""
    out = torch.empty((int(Mcol.numel()), bs, bs), dtype=_F64, device=_dev(Abval))
    call("bilu_isai_compute", nb, bs, _p(_cf(Abval)), _p(_ci(Mbrow)), _p(_ci(Mcol)), int(lower),
         _p(_ci(PairPtr)), _p(_ci(PairPLocal)), _p(_ci(PairSrc)), _p(_cf(Dinv)), _p(out), _s())
    return out


# ------------------------------------------------------------ apply
def bcsr_spmv(MB: int, bs: int, row_ptr, col_ind, val, x, y=None):
    """bcsc2bcsrAndSpMV.h:49 bcsr_spmv: y = M x (FP64; FP32 values take the
    FP32 path with x/y of any float type)."""
    if y is None:
        y = torch.empty(MB * bs, dtype=x.dtype, device=x.device)
    if val.dtype == _F64:
        call("bilu_bcsr_spmv", MB, bs, _p(_ci(row_ptr)), _p(_ci(col_ind)), _p(val.contiguous()),
             _p(x.contiguous()), _p(y), _s())
    else:
        call("bilu_bcsr_spmv_f32", MB, bs, _p(_ci(row_ptr)), _p(_ci(col_ind)),
             _p(_cf(val, _F32)), _p(x.contiguous()), int(x.dtype == _F32), _p(y),
             int(y.dtype == _F32), _s())
    return y


def bcsr_spmm(MB: int, bs: int, row_ptr, col_ind, val, X):
    """Multi-RHS BSR x dense: Y[n, k] = M X[n, k] (k <= 64)."""
    X = _cf(X)
    k = X.shape[1]
    Y = torch.empty_like(X)
    fn = "bilu_bcsr_spmm" if val.dtype == _F64 else "bilu_bcsr_spmm_f32"
    call(fn, MB, bs, k, _p(_ci(row_ptr)), _p(_ci(col_ind)), _p(val.contiguous()), _p(X), _p(Y),
         _s())
    return Y


def bcsr_spmv_transpose(MB: int, bs: int, row_ptr, col_ind, val, x):
    """y = M^T x (adjoint of bcsr_spmv)."""
    y = torch.empty_like(x)
    ws = _ws(lib().bilu_spmv_transpose_ws_bytes(MB, int(col_ind.numel())), x.device)
    call("bilu_bcsr_spmv_transpose", MB, bs, _p(_ci(row_ptr)), _p(_ci(col_ind)), _p(_cf(val)),
         _p(_cf(x)), _p(y), _p(ws), ws.numel(), _s())
    return y


def masked_outer(MB: int, bs: int, row_ptr, col_ind, u, v, scale: float = 1.0, G=None):
    """G[p] (+)= scale * u_I v_J^T on the stored blocks p = (I, J)."""
    acc = G is not None
    if G is None:
        G = torch.empty((int(col_ind.numel()), bs, bs), dtype=_F64, device=u.device)
    call("bilu_masked_outer", MB, bs, _p(_ci(row_ptr)), _p(_ci(col_ind)), _p(_cf(u)), _p(_cf(v)),
         float(scale), int(acc), _p(G), _s())
    return G


def isai_apply(nb: int, bs: int, L, U, b, prec: int = BILU_FP64):
    """main.cu:817-846: y = M_L b, x = M_U y.  L, U: (row, col, val) BCSR."""
    tmp = torch.empty(nb * bs, dtype=_F64 if prec == BILU_FP64 else _F32, device=b.device)
    x = torch.empty_like(b)
    call("bilu_isai_apply", nb, bs, prec, _p(L[0]), _p(L[1]), _p(L[2]), _p(U[0]), _p(U[1]),
         _p(U[2]), _p(_cf(b)), _p(tmp), _p(x), _s())
    return x


# ------------------------------------------------------------ triangular solves
def sptrsv(nb: int, bs: int, row, col, val, b, lower: bool, unit=None, transpose=False):
    """cape_sptrsv.h:8 spTrSolveL (lower) / :55 spTrSolveU (upper), blockwise
    and sync-free on the packed BILU(0).  transpose=True solves L^T / U^T
    over the BCSC view (adjoint)."""
    dev = _dev(b)
    x = torch.empty_like(b)
    nnzb = int(col.numel())
    if transpose:
        ws = _ws(lib().bilu_sptrsv_transpose_ws_bytes(nb, nnzb, bs), dev)
        call("bilu_sptrsv_transpose", nb, bs, _p(_ci(row)), _p(_ci(col)), _p(_cf(val)),
             int(lower), _p(_cf(b)), _p(x), _p(ws), ws.numel(), _s())
        return x
    ws = _ws(lib().bilu_sptrsv_ws_bytes(nb, nnzb), dev)
    if unit is None:
        call("bilu_sptrsv", nb, nnzb, bs, _p(_ci(row)), _p(_ci(col)), _p(_cf(val)), int(lower),
             _p(_cf(b)), _p(x), _p(ws), ws.numel(), _s())
    else:
        call("bilu_sptrsv_ex", nb, nnzb, bs, _p(_ci(row)), _p(_ci(col)), _p(_cf(val)), int(lower),
             int(unit), _p(_cf(b)), _p(x), _p(ws), ws.numel(), _s())
    return x


# ------------------------------------------------------------ verification
def compute_rel_errors(nb: int, bs: int, row, col, val, b, x_true, x):
    """residual_check.h:17 compute_rel_errors_csr on the device ->
    (rel_error_x, rel_residual)."""
    out = (ctypes.c_double * 2)()
    ws = _ws(lib().bilu_rel_errors_ws_bytes(nb, bs), b.device)
    call("bilu_rel_errors", nb, bs, _p(_ci(row)), _p(_ci(col)), _p(_cf(val)), _p(_cf(b)),
         _p(None if x_true is None else _cf(x_true)), _p(_cf(x)), out, _p(ws), ws.numel(), _s())
    return out[0], out[1]


# ------------------------------------------------------------ engine
class _DeviceArray:
    """Zero-copy view of a device pointer owned by the library."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


@dataclass
class SolveResult:
    iters: int
    relres: float
    converged: bool
    history: list
    restarts: int = 0
    inner_steps: int = 0


class Preconditioner:
    """BILU(0)+ISAI engine handle (bilu_ctx): GPU setup of the whole
    preconditioner from a BSR matrix, then preconditioned (F)GMRES solves."""

    def __init__(self, nb: int, bs: int, row, col, val, fp32: bool = True, ilu: bool = False,
                 fp32_inner: bool = False, isai_level: int = 1, schedule: int = -1,
                 stream=None, ilu_fp32: bool = False, nested: bool = False, inner: int = 8):
        self._h = ctypes.c_void_p()
        self.nb, self.bs = nb, bs
        self.stream = stream
        call("bilu_ctx_create", ctypes.byref(self._h), _s(stream))
        call("bilu_ctx_set_isai_level", self._h, isai_level)
        call("bilu_ctx_set_schedule", self._h, schedule)
        call("bilu_ctx_set_inner", self._h, inner)
        self._keep = (row, col, val)
        times = (ctypes.c_double * 4)()
        call("bilu_ctx_setup", self._h, nb, int(col.numel()), bs, _p(_ci(row)), _p(_ci(col)),
             _p(_cf(val)), ((1 << BILU_FP32) if fp32 else 0) | ((1 << BILU_ILU) if ilu else 0)
             | ((1 << BILU_FP32_INNER) if fp32_inner else 0)
             | ((1 << BILU_ILU_FP32) if ilu_fp32 else 0)
             | ((1 << BILU_NESTED) if nested else 0), times)
        self.setup_ms = {"factor": times[0], "patterns": times[1], "isai": times[2],
                         "total": times[3]}

    def close(self):
        if self._h:
            lib().bilu_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get(self, which: int):
        """Copy of a device array built by the handle (see bilu_ctx_get)."""
        ptr, cnt = ctypes.c_void_p(), ctypes.c_longlong(0)
        call("bilu_ctx_get", self._h, which, ctypes.byref(ptr), ctypes.byref(cnt))
        typestr = {0: "<f8", 1: "<i4", 2: "<i4", 3: "<f8", 4: "<i4", 5: "<i4", 6: "<f8",
                   7: "<f4", 8: "<f4"}[which]
        if cnt.value == 0:
            return torch.empty(0, dtype={"<f8": _F64, "<i4": _I32, "<f4": _F32}[typestr],
                               device="cuda")
        return torch.as_tensor(_DeviceArray(ptr.value, cnt.value, typestr), device="cuda").clone()

    def factors(self):
        """(LU values, (Lrow, Lcol, Lval), (Urow, Ucol, Uval)) as tensors."""
        bs = self.bs
        lu = self.get(0).view(-1, bs, bs)
        L = (self.get(1), self.get(2), self.get(3).view(-1, bs, bs))
        U = (self.get(4), self.get(5), self.get(6).view(-1, bs, bs))
        return lu, L, U

    def set_inner(self, k: int):
        """Inner FP32 GMRES steps per outer step of the nested mode."""
        call("bilu_ctx_set_inner", self._h, k)

    def select(self, b, restart: int = 30, cycles: int = 3, tol: float = 1e-10, mask: int = 31):
        """bilu_ctx_select: the preconditioner (BILU_FP64 / BILU_FP32 /
        BILU_ILU / BILU_FP32_INNER / BILU_ILU_FP32 / BILU_NESTED) with the
        best measured residual reduction per second over the last of up to
        `cycles` restart cycles -> (choice, [digits/s])."""
        choice, rate = ctypes.c_int(-1), (ctypes.c_double * 6)()
        call("bilu_ctx_select", self._h, _p(_cf(b)), restart, cycles, tol, mask,
             ctypes.byref(choice), rate)
        nrate = max([4] + [p + 1 for p in (BILU_ILU_FP32, BILU_NESTED) if mask >> p])
        return choice.value, list(rate)[:nrate]

    def solve(self, b, x=None, prec=BILU_FP64, restart: int = 30, tol: float = 1e-10,
              maxit: int = 10000, history: bool = False) -> tuple:
        """prec: BILU_FP64, BILU_FP32, BILU_ILU, BILU_FP32_INNER, BILU_ILU_FP32, BILU_NESTED,
        -1 (none) or "auto" (measured choice by select())."""
        b = _cf(b)
        if prec == "auto":
            prec, _ = self.select(b, restart, tol=tol)
        if x is None:
            x = torch.empty_like(b)
        it, rr = ctypes.c_int(0), ctypes.c_double(0)
        hist = (ctypes.c_double * (maxit + 1))() if history else None
        st = lib().bilu_ctx_solve(self._h, prec, _p(b), _p(x), restart, tol, maxit,
                                  ctypes.byref(it), ctypes.byref(rr), hist)
        if st not in (0, -6):
            raise BiluError("bilu_ctx_solve", st)
        h = list(hist[: it.value + 1]) if history else []
        stats = (ctypes.c_longlong * 4)()
        call("bilu_ctx_stats", self._h, stats)
        inner = ctypes.c_longlong(0)
        call("bilu_ctx_inner_steps", self._h, ctypes.byref(inner))
        return x, SolveResult(it.value, rr.value, st == 0, h, int(stats[1]), int(inner.value))


# ------------------------------------------------------------ host ingest
def read_matrix_market_to_csr(path: str):
    """read_matrix.h:12 read_matrix_market_to_csr (bilu_mtx_read; also
    expands symmetric / skew-symmetric files and reads pattern files)
    -> (nrows, ncols, rowPtr, colInd, vals) as numpy arrays."""
    import numpy as np

    m, n, nnz, bad = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_longlong(0), ctypes.c_longlong(-1)
    p = os.fsencode(path)
    call("bilu_mtx_read", p, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), None, None,
         None, ctypes.byref(bad))
    row = np.zeros(m.value + 1, np.int32)
    col = np.zeros(max(nnz.value, 1), np.int32)
    val = np.zeros(max(nnz.value, 1), np.float64)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    call("bilu_mtx_read", p, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), P(row), P(col),
         P(val), ctypes.byref(bad))
    return m.value, n.value, row, col[: nnz.value], val[: nnz.value]


def bsr_save(path: str, nb: int, bs: int, rowptr, colind, val):
    """Write a BSR matrix (numpy arrays) to the binary format of bilu_bsr_save."""
    import numpy as np

    row = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(colind, np.int32)
    v = np.ascontiguousarray(val, np.float64)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    call("bilu_bsr_save", os.fsencode(path), nb, int(col.shape[0]), bs, P(row), P(col), P(v))


def bsr_load(path: str):
    """Read a file written by bsr_save -> (nb, bs, rowptr, colind, val[nnzb, bs, bs])."""
    import numpy as np

    nb, nnzb, bs = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    p = os.fsencode(path)
    call("bilu_bsr_load", p, ctypes.byref(nb), ctypes.byref(nnzb), ctypes.byref(bs), None, None,
         None)
    row = np.zeros(nb.value + 1, np.int32)
    col = np.zeros(max(nnzb.value, 1), np.int32)
    val = np.zeros(max(nnzb.value * bs.value * bs.value, 1), np.float64)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    call("bilu_bsr_load", p, ctypes.byref(nb), ctypes.byref(nnzb), ctypes.byref(bs), P(row),
         P(col), P(val))
    k = nnzb.value
    return nb.value, bs.value, row, col[:k], val[: k * bs.value * bs.value].reshape(k, bs.value,
                                                                                  bs.value)


def block_diagonal_union(mats):
    """Concatenate BSR systems into one block-diagonal BSR matrix with global
    column indices -> (sys_ptr[S+1], rowptr, colind, val[nnzb, bs, bs])."""
    import numpy as np

    sys_ptr = np.zeros(len(mats) + 1, np.int32)
    rows, cols, vals = [np.zeros(1, np.int64)], [], []
    off_r, off_nz = 0, 0
    for i, A in enumerate(mats):
        rows.append(A.rowptr[1:].astype(np.int64) + off_nz)
        cols.append(A.colind.astype(np.int64) + off_r)
        vals.append(A.val)
        off_r += A.nb
        off_nz += A.nnzb
        sys_ptr[i + 1] = off_r
    return (sys_ptr, np.concatenate(rows).astype(np.int32), np.concatenate(cols).astype(np.int32),
            np.concatenate(vals))


class Batch:
    """Many uneven systems with k right-hand sides each (bilu_batch): one
    setup on the block-diagonal union, then per-(system, rhs) FGMRES with the
    FP32 ISAI apply as BSR x dense SpMM, graph-replayed Arnoldi steps and an
    autotuned SpMM tile."""

    def __init__(self, mats, stream=None):
        import numpy as np

        self._h = ctypes.c_void_p()
        self.bs = mats[0].bs
        sys_ptr, rowptr, colind, val = block_diagonal_union(mats)
        self.sys_ptr = sys_ptr
        self.S = len(mats)
        self.nb = int(sys_ptr[-1])
        self.row = torch.from_numpy(rowptr).cuda()
        self.col = torch.from_numpy(colind).cuda()
        self.val = torch.from_numpy(val).cuda()
        call("bilu_batch_create", ctypes.byref(self._h), _s(stream))
        times = (ctypes.c_double * 4)()
        call("bilu_batch_setup", self._h, self.S, sys_ptr.ctypes.data_as(ctypes.c_void_p),
             int(colind.shape[0]), self.bs, _p(self.row), _p(self.col), _p(self.val), times)
        self.setup_ms = list(times)
        self._np = np

    def set_schedule(self, persistent: bool):
        """One cooperative launch per Arnoldi step (True, the default) or a
        graph of per-phase launches (False); the results are identical."""
        call("bilu_batch_set_schedule", self._h, int(persistent))

    def close(self):
        if self._h:
            lib().bilu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, B, restart: int = 30, tol: float = 1e-10, maxit: int = 10000,
              mem_budget: int = 0):
        """B: [n, k] FP64 CUDA tensor.  Returns X, iters[S, k], relres[S, k],
        stats (waves, graph launches, pair-steps, solve ms)."""
        np = self._np
        B = _cf(B)
        k = B.shape[1]
        X = torch.empty_like(B)
        iters = np.zeros(self.S * k, np.int32)
        relres = np.zeros(self.S * k)
        stats = (ctypes.c_double * 4)()
        call("bilu_batch_solve", self._h, k, _p(B), _p(X), restart, tol, maxit,
             ctypes.c_longlong(mem_budget), iters.ctypes.data_as(ctypes.c_void_p),
             relres.ctypes.data_as(ctypes.c_void_p), stats)
        return X, iters.reshape(self.S, k), relres.reshape(self.S, k), list(stats)

    def tuning(self):
        cfg = (ctypes.c_int * 3)()
        ms = (ctypes.c_double * 6)()
        call("bilu_batch_tuning", self._h, cfg, ms)
        return list(cfg), list(ms)


def solve_host(nb: int, bs: int, row, col, val, b, prec: int = BILU_FP64, restart: int = 30,
               tol: float = 1e-10, maxit: int = 10000):
    """End-to-end call with host (numpy) buffers: H2D, setup, solve, D2H."""
    import numpy as np

    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.empty_like(b)
    it, rr = ctypes.c_int(0), ctypes.c_double(0)
    times = (ctypes.c_double * 4)()
    st = lib().bilu_solve_host(nb, int(col.shape[0]), bs, row.ctypes.data, col.ctypes.data,
                               val.ctypes.data, b.ctypes.data, x.ctypes.data, prec, restart, tol,
                               maxit, ctypes.byref(it), ctypes.byref(rr), times, _s())
    if st not in (0, -6):
        raise BiluError("bilu_solve_host", st)
    return x, SolveResult(it.value, rr.value, st == 0, []), list(times)
