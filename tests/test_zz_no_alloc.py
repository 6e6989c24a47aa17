"""The allocation-free triangular solve (bilu_sptrsv_noalloc), for callers
that cannot allocate device memory (hosts whose device memory belongs to a
fixed arena or budget, plugins restricted to the buffers they are given).

Called through the C ABI and compared with the CPU oracle's block triangular
solves (orc_sptrsv_lower / orc_sptrsv_upper on the oracle's BILU(0) factor),
two calls in a row (the shared scratch array keeps the previous call's
contents, so the second call checks that everything that must start at zero
is re-initialised), within the 1e-12 relative tolerance the other
triangular-solve tests use, and beside the workspace-taking bilu_sptrsv.
Edge cases: nb = 0, a block row without its diagonal block, b aliasing x,
and a size beyond the fixed array.  This file is collected last so a
stop-at-first-failure run has run every other test."""
import ctypes

import numpy as np
import pytest

from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu


def _relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _noalloc(L, nb, bs, row, col, val, lower, b, x):
    import torch

    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    return L.bilu_sptrsv_noalloc(nb, bs, ptr(row), ptr(col), ptr(val), lower, ptr(b), ptr(x),
                                 stream)


def test_noalloc_sptrsv_matches_oracle(cuda, orc):
    import torch

    from isai_kernel_gb300 import _lib, api

    L = _lib.lib()
    cases = [gen.convdiff3d(10, bs=4, seed=0), gen.laplace2d(12, bs=5, seed=3),
             gen.powerlaw(300, bs=8, seed=1, kmax=30)]
    for A in cases:
        LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
        row = torch.from_numpy(A.rowptr).to(cuda)
        col = torch.from_numpy(A.colind).to(cuda)
        lu = torch.from_numpy(LU).to(cuda)
        for call in range(2):
            b_np = gen.rhs(A.n, 10 + call)
            b = torch.from_numpy(b_np).to(cuda)
            for lower in (1, 0):
                if lower:
                    ref = orc.sptrsv_lower(A.nb, A.bs, A.rowptr, A.colind, LU, b_np)
                else:
                    ref = orc.sptrsv_upper(A.nb, A.bs, A.rowptr, A.colind, LU, b_np)
                x = torch.full_like(b, float("nan"))
                st = _noalloc(L, A.nb, A.bs, row, col, lu, lower, b, x)
                assert st == 0, _lib.STATUS.get(st, st)
                torch.cuda.synchronize()
                got = x.cpu().numpy()
                assert _relerr(got, ref) <= 1e-12, (A.nb, A.bs, call, lower)
                # and the workspace-taking solve agrees with it
                ws = api.sptrsv(A.nb, A.bs, row, col, lu, b, lower=bool(lower))
                assert _relerr(got, ws.cpu().numpy()) <= 1e-12


def test_noalloc_edge_cases(cuda, orc):
    import torch

    from isai_kernel_gb300 import _lib

    L = _lib.lib()
    # nb = 0: nothing to do, nothing touched
    assert _noalloc(L, 0, 4, None, None, None, 1, None, None) == 0
    # a block row whose diagonal block is not stored: BILU_ERR_PATTERN
    A = gen.laplace2d(6, bs=4, seed=0)
    keep = np.ones(A.nnzb, dtype=bool)
    r = 7
    for p in range(A.rowptr[r], A.rowptr[r + 1]):
        if A.colind[p] == r:
            keep[p] = False
    cnt = np.array([keep[A.rowptr[i]:A.rowptr[i + 1]].sum() for i in range(A.nb)])
    row_np = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    col_np = A.colind[keep].astype(np.int32)
    val_np = A.val[keep]
    row = torch.from_numpy(row_np).to(cuda)
    col = torch.from_numpy(col_np).to(cuda)
    val = torch.from_numpy(np.ascontiguousarray(val_np)).to(cuda)
    b = torch.from_numpy(gen.rhs(A.n, 1)).to(cuda)
    x = torch.empty_like(b)
    for lower in (1, 0):
        assert _noalloc(L, A.nb, 4, row, col, val, lower, b, x) == -2  # BILU_ERR_PATTERN
    # b and x in the same buffer: BILU_ERR_ARG
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row = torch.from_numpy(A.rowptr).to(cuda)
    col = torch.from_numpy(A.colind).to(cuda)
    lu = torch.from_numpy(LU).to(cuda)
    assert _noalloc(L, A.nb, 4, row, col, lu, 1, b, b) == -1
    # a good call after the failed ones still matches the oracle
    b_np = gen.rhs(A.n, 2)
    b = torch.from_numpy(b_np).to(cuda)
    assert _noalloc(L, A.nb, 4, row, col, lu, 0, b, x) == 0
    torch.cuda.synchronize()
    ref = orc.sptrsv_upper(A.nb, A.bs, A.rowptr, A.colind, LU, b_np)
    assert _relerr(x.cpu().numpy(), ref) <= 1e-12


def test_noalloc_rejects_oversize(cuda):
    import torch

    from isai_kernel_gb300 import _lib

    L = _lib.lib()
    nmax = L.bilu_sptrsv_noalloc_max_rows()
    assert nmax == 262144
    dummy = torch.zeros(8, dtype=torch.float64, device=cuda)
    dummy2 = torch.zeros(8, dtype=torch.float64, device=cuda)
    p = ctypes.c_void_p(dummy.data_ptr())
    q = ctypes.c_void_p(dummy2.data_ptr())
    st = L.bilu_sptrsv_noalloc(nmax + 1, 4, p, p, p, 1, p, q, None)
    assert st == -7  # BILU_ERR_WORKSPACE: beyond the fixed scratch array
