"""The allocation-free triangular solve (bilu_sptrsv_noalloc), for callers
that cannot allocate device memory (graph capture, fixed memory arenas,
plugins restricted to the buffers they are given).

Called through the C ABI and compared with the workspace-taking
bilu_sptrsv on the same inputs, two calls in a row (the shared scratch array
keeps the previous call's contents, so the second call checks that
everything that must start at zero is re-initialised), within the 1e-12
relative tolerance the other triangular-solve tests use.  This file is
collected last so a stop-at-first-failure run has run every other test."""
import ctypes

import numpy as np
import pytest

from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu


def _relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_noalloc_sptrsv_matches_workspace_version(cuda, orc):
    import torch

    from isai_kernel_gb300 import _lib, api

    L = _lib.lib()
    cases = [gen.convdiff3d(10, bs=4, seed=0), gen.powerlaw(300, bs=8, seed=1, kmax=30)]
    for A in cases:
        LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
        dev = cuda
        row = torch.from_numpy(A.rowptr).to(dev)
        col = torch.from_numpy(A.colind).to(dev)
        lu = torch.from_numpy(LU).to(dev)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for call in range(2):
            b = torch.from_numpy(gen.rhs(A.n, 10 + call)).to(dev)
            for lower in (1, 0):
                ref = api.sptrsv(A.nb, A.bs, row, col, lu, b, lower=bool(lower))
                x = torch.full_like(b, float("nan"))
                st = L.bilu_sptrsv_noalloc(A.nb, A.bs, ctypes.c_void_p(row.data_ptr()),
                                           ctypes.c_void_p(col.data_ptr()),
                                           ctypes.c_void_p(lu.data_ptr()), lower,
                                           ctypes.c_void_p(b.data_ptr()),
                                           ctypes.c_void_p(x.data_ptr()), stream)
                assert st == 0, _lib.STATUS.get(st, st)
                torch.cuda.synchronize()
                assert _relerr(x.cpu().numpy(), ref.cpu().numpy()) <= 1e-12


def test_noalloc_rejects_oversize(cuda):
    import torch

    from isai_kernel_gb300 import _lib

    L = _lib.lib()
    nmax = L.bilu_sptrsv_noalloc_max_rows()
    assert nmax == 262144
    dummy = torch.zeros(8, dtype=torch.float64, device=cuda)
    p = ctypes.c_void_p(dummy.data_ptr())
    st = L.bilu_sptrsv_noalloc(nmax + 1, 4, p, p, p, 1, p, p, None)
    assert st == -7  # BILU_ERR_WORKSPACE: beyond the fixed scratch array
