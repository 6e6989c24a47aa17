"""The sync-free GPU BILU(0) and block triangular solves against cuSPARSE
bsrilu02 / bsrsv2 called with the reference's settings (bsrilu.h:20-66,
BILU_cusparse.h:110-224): factors and solutions within 1e-12 relative, and
the same zero pivot."""
import ctypes
import os

import numpy as np
import pytest

from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(os.path.dirname(HERE), "oracle", "libcusparse_ref.so")


@pytest.fixture(scope="module")
def cusp(cuda):
    if not os.path.exists(LIB):
        pytest.fail("oracle/libcusparse_ref.so not built (build() runs `make -C oracle cusparse`)")
    L = ctypes.CDLL(LIB)
    for f in (L.cusp_bsrilu02, L.cusp_bsrsv2):
        f.restype = ctypes.c_int
    return L


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


CASES = [lambda: gen.laplace2d(24, bs=4, seed=0), lambda: gen.convdiff3d(12, bs=4, seed=1),
         lambda: gen.powerlaw(400, bs=8, seed=2, kmax=40), lambda: gen.laplace2d(10, bs=5, seed=3)]


@pytest.mark.parametrize("mk", CASES)
def test_bilu0_and_solves_match_cusparse(cuda, cusp, mk):
    import torch

    from isai_kernel_gb300 import api

    A = mk()
    row = torch.from_numpy(A.rowptr).to(cuda)
    col = torch.from_numpy(A.colind).to(cuda)
    ours = torch.from_numpy(A.val).to(cuda).contiguous()
    theirs = ours.clone()
    assert api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, row, col, ours) == -1
    zp = ctypes.c_int(0)
    ms = (ctypes.c_float * 2)()
    assert cusp.cusp_bsrilu02(A.nb, A.nnzb, A.bs, P(row), P(col), P(theirs), ctypes.byref(zp),
                              ms) == 0
    assert zp.value == -1
    assert relerr(ours.cpu().numpy(), theirs.cpu().numpy()) < 1e-12
    b = torch.from_numpy(gen.rhs(A.n, 5)).to(cuda)
    for lower in (True, False):
        x = api.sptrsv(A.nb, A.bs, row, col, ours, b, lower=lower)
        xr = torch.empty_like(b)
        assert cusp.cusp_bsrsv2(A.nb, A.nnzb, A.bs, P(row), P(col), P(theirs), int(lower), P(b),
                                P(xr), 1, ms) == 0
        torch.cuda.synchronize()
        assert relerr(x.cpu().numpy(), xr.cpu().numpy()) < 1e-12


def test_zero_pivot_matches_cusparse(cuda, cusp):
    import torch

    from isai_kernel_gb300 import api

    A = gen.laplace2d(6, bs=4, seed=0)
    d = [p for p in range(A.rowptr[0], A.rowptr[1]) if A.colind[p] == 0][0]
    A.val[d][2, :] = 0.0
    row = torch.from_numpy(A.rowptr).to(cuda)
    col = torch.from_numpy(A.colind).to(cuda)
    ours = torch.from_numpy(A.val).to(cuda).contiguous()
    theirs = ours.clone()
    info = api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, row, col, ours)
    zp = ctypes.c_int(0)
    ms = (ctypes.c_float * 2)()
    assert cusp.cusp_bsrilu02(A.nb, A.nnzb, A.bs, P(row), P(col), P(theirs), ctypes.byref(zp),
                              ms) == 0
    assert info == zp.value == 0
