"""ctypes wrapper of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and the CPU-baseline leg of bench.py use this
module, and only as the checker.  Each function restates the reference step
named in its docstring (file:line in gmfff/isai_kernel).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build() -> str:
    """Compile liboracle.so with the committed Makefile (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return os.path.join(HERE, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        src = os.path.join(HERE, "bilu_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = ctypes.CDLL(path)
        _LIB.orc_num_threads.restype = ctypes.c_int
    return _LIB


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _call(name, *args):
    f = getattr(lib(), name)
    f.restype = ctypes.c_int
    return f(*[a.ctypes.data_as(ctypes.c_void_p) if isinstance(a, np.ndarray) else a
               for a in args])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(ctypes.c_int(n))


def num_threads() -> int:
    return lib().orc_num_threads()


class OracleError(RuntimeError):
    def __init__(self, name, code, info=None):
        super().__init__(f"{name} failed with status {code} ({info})")
        self.code = code
        self.info = info


def _chk(name, st, info=None):
    if st != 0:
        raise OracleError(name, st, info)


def csr_to_bsr(n, bs, row, col, val):
    """csr2bsr.h:14 csr_to_bsr5 -> (rowptr, colind, val[nnzb,bs,bs])."""
    row, col, val = _i(row), _i(col), _d(val)
    nb = n // bs
    brow = np.zeros(nb + 1, np.int32)
    _chk("csr_to_bsr_count", _call("orc_csr_to_bsr_count", n, bs, row, col, brow))
    nnzb = int(brow[-1])
    bcol = np.zeros(nnzb, np.int32)
    bval = np.zeros((nnzb, bs, bs))
    _chk("csr_to_bsr_fill", _call("orc_csr_to_bsr_fill", n, bs, row, col, val, brow, bcol, bval))
    return brow, bcol, bval


def isai_pattern(nb, Arow, Acol, lower):
    """isai_bsr.h:246 build_bcsc_pattern_from_bsr_scalarILU -> (Mptr, Mind)."""
    Arow, Acol = _i(Arow), _i(Acol)
    mp = np.zeros(nb + 1, np.int32)
    _chk("isai_pattern_count", _call("orc_isai_pattern_count", nb, Arow, Acol, int(lower), mp))
    mi = np.zeros(int(mp[-1]), np.int32)
    _chk("isai_pattern_fill", _call("orc_isai_pattern_fill", nb, Arow, Acol, int(lower), mp, mi))
    return mp, mi


def pattern_product(nb, Xrow, Xcol, Arow, Acol):
    """Symbolic C = pattern(X A), rows sorted and distinct -> (Crow, Ccol)."""
    Xrow, Xcol, Arow, Acol = _i(Xrow), _i(Xcol), _i(Arow), _i(Acol)
    cr = np.zeros(nb + 1, np.int32)
    f = lib().orc_pattern_product
    f.restype = ctypes.c_int
    _chk("pattern_product", f(nb, _ptr(Xrow), _ptr(Xcol), _ptr(Arow), _ptr(Acol), _ptr(cr), None))
    cc = np.zeros(int(cr[-1]), np.int32)
    _chk("pattern_product", f(nb, _ptr(Xrow), _ptr(Xcol), _ptr(Arow), _ptr(Acol), _ptr(cr),
                              _ptr(cc)))
    return cr, cc


def pattern_power(nb, Arow, Acol, k):
    """pattern(A^k) as (rowptr, colind) (k = 1: A's own pattern)."""
    pr, pc = _i(Arow), _i(Acol)
    for _ in range(k - 1):
        pr, pc = pattern_product(nb, pr, pc, Arow, Acol)
    return pr, pc


def tri_pattern(nb, Arow, Acol, lower):
    """bcsc2bcsr.h:11 build_triangular_bcsr_pattern_from_A -> (Trow, Tcol)."""
    Arow, Acol = _i(Arow), _i(Acol)
    tr = np.zeros(nb + 1, np.int32)
    _call("orc_tri_pattern_count", nb, Arow, Acol, int(lower), tr)
    tc = np.zeros(int(tr[-1]), np.int32)
    _call("orc_tri_pattern_fill", nb, Arow, Acol, int(lower), tr, tc)
    return tr, tc


def map_bcsc2bcsr(nb, cptr, cind, rptr, rcol):
    """bcsc2bcsr.h:32 build_map_bcsc2bcsr_host."""
    m = np.zeros(int(cptr[-1]), np.int32)
    br, bc = ctypes.c_int(-1), ctypes.c_int(-1)
    f = lib().orc_map_bcsc2bcsr
    f.restype = ctypes.c_int
    st = f(nb, _ptr(_i(cptr)), _ptr(_i(cind)), _ptr(_i(rptr)), _ptr(_i(rcol)), _ptr(m),
           ctypes.byref(br), ctypes.byref(bc))
    _chk("map_bcsc2bcsr", st, (br.value, bc.value))
    return m


def reorder_bcsc_to_bcsr(bs, mp, src):
    """bcsc2bcsr.h:63 reorder_bcsc_val_to_bcsr_bs5."""
    src = _d(src)
    dst = np.zeros_like(src)
    _call("orc_reorder_bcsc_to_bcsr", int(mp.shape[0]), bs, _i(mp), src, dst)
    return dst


def bcsc_to_bcsr(mb, nbcol, bs, cptr, cind, cval):
    """bcsc2bcsrAndSpMV.h:76 bcsc_to_bcsr (deterministic row order)."""
    nnzb = int(cptr[-1])
    rp = np.zeros(mb + 1, np.int32)
    ci = np.zeros(nnzb, np.int32)
    v = np.zeros((nnzb, bs, bs))
    _chk("bcsc_to_bcsr", _call("orc_bcsc_to_bcsr", mb, nbcol, bs, _i(cptr), _i(cind),
                               _d(cval), rp, ci, v))
    return rp, ci, v


def bsr_to_csr(mb, bs, Arow, Acol, Aval):
    """bsr2csr.h:19 bsr2csr_cusparse (row direction)."""
    nnzb = int(Arow[-1])
    rp = np.zeros(mb * bs + 1, np.int32)
    ci = np.zeros(nnzb * bs * bs, np.int32)
    v = np.zeros(nnzb * bs * bs)
    _call("orc_bsr_to_csr", mb, bs, _i(Arow), _i(Acol), _d(Aval), rp, ci, v)
    return rp, ci, v


def bsrilu0(nb, bs, Arow, Acol, Aval):
    """bsrilu.h:20 bsrilu02_inplace -> (packed LU values, zero_pivot or -1)."""
    v = _d(Aval).copy()
    zp = ctypes.c_int(-1)
    f = lib().orc_bsrilu0
    f.restype = ctypes.c_int
    st = f(nb, bs, _ptr(_i(Arow)), _ptr(_i(Acol)), _ptr(v), ctypes.byref(zp))
    if st not in (0, -3):
        _chk("bsrilu0", st, zp.value)
    return v, zp.value


def csr_ilu0(n, row, col, val):
    v = _d(val).copy()
    zp = ctypes.c_int(-1)
    f = lib().orc_csr_ilu0
    f.restype = ctypes.c_int
    st = f(n, _ptr(_i(row)), _ptr(_i(col)), _ptr(v), ctypes.byref(zp))
    if st not in (0, -3):
        _chk("csr_ilu0", st, zp.value)
    return v, zp.value


def dinv(nb, bs, Arow, Acol, Aval, lower):
    """isai_bsr.h:91/126 build_DinvL/DinvU_from_BSR5_kernel_fix."""
    out = np.zeros((nb, bs, bs))
    _chk("dinv", _call("orc_dinv", nb, bs, _i(Arow), _i(Acol), _d(Aval), int(lower), out))
    return out


def pairs_lower(nb, Arow, Acol, Mptr, Mind):
    """isai_bsr.h:1378/1427 count/fill_pairs_lower_kernel_v2 + exclusive scan
    (main.cu:684) -> (PairPtr[Mnnz+1], PairPLocal, PairSrc)."""
    Arow, Acol, Mptr, Mind = _i(Arow), _i(Acol), _i(Mptr), _i(Mind)
    mnnz = int(Mptr[-1])
    cnt = np.zeros(mnnz, np.int32)
    _call("orc_count_pairs_lower", nb, Arow, Acol, Mptr, Mind, cnt)
    pp = np.zeros(mnnz + 1, np.int32)
    np.cumsum(cnt, out=pp[1:])
    pl = np.zeros(int(pp[-1]), np.int32)
    ps = np.zeros(int(pp[-1]), np.int32)
    _call("orc_fill_pairs_lower", nb, Arow, Acol, Mptr, Mind, pp, pl, ps)
    return pp, pl, ps


def isai_lower(nb, bs, Aval, Mptr, Mind, pp, pl, ps, DinvL):
    """isai_bsr.h:288 isai_lower_* -> M_L values in BCSC order."""
    out = np.zeros((int(Mptr[-1]), bs, bs))
    _call("orc_isai_lower", nb, bs, _d(Aval), _i(Mptr), _i(Mind), _i(pp), _i(pl), _i(ps),
          _d(DinvL), out)
    return out


def isai_upper(nb, bs, Arow, Acol, Aval, Mptr, Mind, DinvU):
    """isai_bsr.h:161 isai_upper_bsr5_warpcol_with_Dinv_kernel."""
    out = np.zeros((int(Mptr[-1]), bs, bs))
    _call("orc_isai_upper", nb, bs, _i(Arow), _i(Acol), _d(Aval), _i(Mptr), _i(Mind),
          _d(DinvU), out)
    return out


def bcsr_spmv(mb, bs, row, col, val, x):
    """bcsc2bcsrAndSpMV.h:119 cpu_bcsr_spmv."""
    y = np.zeros(mb * bs)
    _call("orc_bcsr_spmv", mb, bs, _i(row), _i(col), _d(val), _d(x), y)
    return y


def bcsr_spmv_f32(mb, bs, row, col, val, x):
    y = np.zeros(mb * bs, np.float32)
    _call("orc_bcsr_spmv_f32", mb, bs, _i(row), _i(col),
          np.ascontiguousarray(val, np.float32), np.ascontiguousarray(x, np.float32), y)
    return y


def sptrsv_lower(nb, bs, row, col, val, b):
    """cape_sptrsv.h:8 spTrSolveL semantics, blockwise (unit lower)."""
    x = np.zeros(nb * bs)
    _chk("sptrsv_lower", _call("orc_sptrsv_lower", nb, bs, _i(row), _i(col), _d(val), _d(b), x))
    return x


def sptrsv_upper(nb, bs, row, col, val, b):
    """cape_sptrsv.h:55 spTrSolveU semantics, blockwise."""
    x = np.zeros(nb * bs)
    _chk("sptrsv_upper", _call("orc_sptrsv_upper", nb, bs, _i(row), _i(col), _d(val), _d(b), x))
    return x


def rel_errors(n, row, col, val, b, x_true, x):
    """residual_check.h:16 compute_rel_errors_csr -> (rel_err, rel_res)."""
    e, r = ctypes.c_double(0), ctypes.c_double(0)
    f = lib().orc_rel_errors_csr
    f.restype = ctypes.c_int
    xt = None if x_true is None else _d(x_true)
    f(n, _ptr(_i(row)), _ptr(_i(col)), _ptr(_d(val)), _ptr(_d(b)), _ptr(xt), _ptr(_d(x)),
      ctypes.byref(e), ctypes.byref(r))
    return e.value, r.value


def gmres(A, L, U, b, precond=1, restart=30, tol=1e-10, maxit=3000):
    """Restarted right-preconditioned (F)GMRES(m) with modified Gram-Schmidt (no counterpart
    in the reference).  A, L, U: (rowptr, colind, val) triples in BCSR.
    Returns (x, iters, relres, history, status)."""
    nb = A[0].shape[0] - 1
    bs = A[2].shape[1]
    x = np.zeros(nb * bs)
    it, rr = ctypes.c_int(0), ctypes.c_double(0)
    hist = np.zeros(maxit + 1)
    L = L if L is not None else A
    U = U if U is not None else A
    f = lib().orc_gmres
    f.restype = ctypes.c_int
    st = f(nb, bs, _ptr(_i(A[0])), _ptr(_i(A[1])), _ptr(_d(A[2])), _ptr(_i(L[0])),
           _ptr(_i(L[1])), _ptr(_d(L[2])), _ptr(_i(U[0])), _ptr(_i(U[1])), _ptr(_d(U[2])),
           precond, _ptr(_d(b)), _ptr(x), restart, ctypes.c_double(tol), maxit,
           ctypes.byref(it), ctypes.byref(rr), _ptr(hist))
    return x, it.value, rr.value, hist[: it.value + 1], st


def gmres_nested(A, L, U, b, inner=30, restart=30, tol=1e-10, maxit=3000):
    """FP64 outer FGMRES(restart) whose preconditioner is `inner` steps of FP32
    ISAI-preconditioned GMRES on the FP32-stored A (the nested, GMRES-IR mode;
    no counterpart in the reference).  Returns (x, outer iterations, inner
    steps in total, relres, history, status)."""
    nb = A[0].shape[0] - 1
    bs = A[2].shape[1]
    x = np.zeros(nb * bs)
    it, rr, tot = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_longlong(0)
    hist = np.zeros(maxit + 1)
    f = lib().orc_gmres_ex
    f.restype = ctypes.c_int
    st = f(nb, bs, _ptr(_i(A[0])), _ptr(_i(A[1])), _ptr(_d(A[2])), _ptr(_i(L[0])),
           _ptr(_i(L[1])), _ptr(_d(L[2])), _ptr(_i(U[0])), _ptr(_i(U[1])), _ptr(_d(U[2])),
           5, inner, _ptr(_d(b)), _ptr(x), restart, ctypes.c_double(tol), maxit,
           ctypes.byref(it), ctypes.byref(tot), ctypes.byref(rr), _ptr(hist))
    return x, it.value, tot.value, rr.value, hist[: it.value + 1], st


def isai_setup(A, level=1):
    """Full oracle setup on a BSRMatrix: BILU(0), patterns, pairs, Dinv,
    ISAI-L/U and BCSR reorder.  level k > 1: ISAI(k), the M patterns taken
    from pattern(A^k).  Returns a dict of every intermediate."""
    nb, bs = A.nb, A.bs
    LU, zp = bsrilu0(nb, bs, A.rowptr, A.colind, A.val)
    out = {"LU": LU, "zero_pivot": zp}
    Pr, Pc = pattern_power(nb, A.rowptr, A.colind, level)
    for lower, tag in ((True, "L"), (False, "U")):
        mp, mi = isai_pattern(nb, Pr, Pc, lower)
        tr, tc = tri_pattern(nb, Pr, Pc, lower)
        mp_map = map_bcsc2bcsr(nb, mp, mi, tr, tc)
        D = dinv(nb, bs, A.rowptr, A.colind, LU, lower)
        if lower:
            pp, pl, ps = pairs_lower(nb, A.rowptr, A.colind, mp, mi)
            M = isai_lower(nb, bs, LU, mp, mi, pp, pl, ps, D)
            out.update(PairPtr=pp, PairPLocal=pl, PairSrc=ps)
        else:
            M = isai_upper(nb, bs, A.rowptr, A.colind, LU, mp, mi, D)
        out.update({f"Mptr{tag}": mp, f"Mind{tag}": mi, f"Trow{tag}": tr, f"Tcol{tag}": tc,
                    f"map{tag}": mp_map, f"Dinv{tag}": D, f"Mcsc{tag}": M,
                    f"Mcsr{tag}": reorder_bcsc_to_bcsr(bs, mp_map, M)})
    return out
