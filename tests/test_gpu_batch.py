"""Batched multi-RHS solves (bilu_batch): uneven 2D 5-point 4-DOF systems,
several right-hand sides each, in one block-diagonal setup.  Every
(system, rhs) pair must converge to 1e-10 true relative residual, take the
iteration count of the single-RHS mixed-precision solve of the same system
within +-2 (FP32 ISAI apply, different FP32 summation order), give the same
answer whether the batch runs in one wave or in several and whether a step
is one cooperative launch or a graph of per-phase launches (bit-identical),
and the SpMM of the apply must match the column-wise SpMV."""
import numpy as np
import pytest

from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu


def _mats():
    sides = [6, 9, 12, 7, 10, 8]
    return [gen.laplace2d(s, bs=4, seed=10 + i) for i, s in enumerate(sides)]


def test_batch_matches_single_rhs(cuda, orc):
    import torch

    from isai_kernel_gb300 import api

    mats = _mats()
    k = 4
    B_np = np.concatenate([gen.rhs(A.n, 100 + i, k=k) for i, A in enumerate(mats)])
    bt = api.Batch(mats)
    X, iters, relres, stats = bt.solve(torch.from_numpy(B_np).cuda(), maxit=3000)
    assert stats[0] == 1 and stats[1] > 0
    assert np.all(relres <= 1e-10), relres
    Xn = X.cpu().numpy()
    off = 0
    for s, A in enumerate(mats):
        D = A.to_dense()
        row, col, val = (torch.from_numpy(a).cuda() for a in (A.rowptr, A.colind, A.val))
        P = api.Preconditioner(A.nb, A.bs, row, col, val)
        for c in range(k):
            b = B_np[off:off + A.n, c]
            x = Xn[off:off + A.n, c]
            assert np.linalg.norm(b - D @ x) / np.linalg.norm(b) <= 1.01e-10
            _, res = P.solve(torch.from_numpy(np.ascontiguousarray(b)).cuda(), prec=1, maxit=3000)
            assert abs(res.iters - int(iters[s, c])) <= 2, (s, c, res.iters, iters[s, c])
        P.close()
        off += A.n
    cfg, ms = bt.tuning()
    assert cfg[0] in (1, 2, 4) and cfg[1] in (1, 2, 4) and all(t > 0 for t in ms)
    # several waves (tiny memory budget) give the same bits
    X2, iters2, relres2, stats2 = bt.solve(torch.from_numpy(B_np).cuda(), maxit=3000,
                                           mem_budget=1 << 20)
    assert stats2[0] > 1
    assert np.array_equal(iters2, iters) and np.array_equal(X2.cpu().numpy(), Xn)
    # the graph of per-phase launches gives the bits of the one-launch step
    bt.set_schedule(False)
    X3, iters3, relres3, stats3 = bt.solve(torch.from_numpy(B_np).cuda(), maxit=3000)
    assert np.array_equal(iters3, iters) and np.array_equal(X3.cpu().numpy(), Xn)
    assert np.array_equal(relres3, relres)
    bt.close()


def test_batch_rejects_coupled_systems(cuda):
    import torch

    from isai_kernel_gb300 import _lib, api

    mats = _mats()[:2]
    sys_ptr, rowptr, colind, val = api.block_diagonal_union(mats)
    colind = colind.copy()
    colind[rowptr[1] - 1] = sys_ptr[1] + 1  # row 0 reaches into system 1
    h = api.ctypes.c_void_p()
    api.call("bilu_batch_create", api.ctypes.byref(h), api._s())
    row, col, v = (torch.from_numpy(a).cuda() for a in (rowptr, colind, val))
    st = _lib.lib().bilu_batch_setup(h, 2, sys_ptr.ctypes.data_as(api.ctypes.c_void_p),
                                     int(colind.shape[0]), 4, api._p(row), api._p(col), api._p(v),
                                     None)
    assert st == -2
    _lib.lib().bilu_batch_destroy(h)


def test_batch_matches_oracle_per_pair(cuda, orc):
    """Every (system, rhs) pair of the batch against the oracle's own
    mixed-precision FGMRES(30) (FP32-stored ISAI, FP32 accumulation, FP64
    operator, orthogonalisation and restarts) on that system and column:
    iteration counts within +-2 (FP32 summation order differs), x within
    1e-8 of the oracle's FP64 GMRES solution of the same pair."""
    import torch

    from isai_kernel_gb300 import api

    mats = [gen.laplace2d(s, bs=4, seed=40 + i) for i, s in enumerate([5, 11, 8, 13, 6])]
    k = 3
    B_np = np.concatenate([gen.rhs(A.n, 200 + i, k=k) for i, A in enumerate(mats)])
    bt = api.Batch(mats)
    X, iters, relres, stats = bt.solve(torch.from_numpy(B_np).cuda(), maxit=3000)
    bt.close()
    assert np.all(relres <= 1e-10), relres
    Xn = X.cpu().numpy()
    off = 0
    for s, A in enumerate(mats):
        S = orc.isai_setup(A)
        Ab = (A.rowptr, A.colind, A.val)
        Lo = (S["TrowL"], S["TcolL"], S["McsrL"])
        Uo = (S["TrowU"], S["TcolU"], S["McsrU"])
        for c in range(k):
            b = np.ascontiguousarray(B_np[off:off + A.n, c])
            _, itm, _, _, stm = orc.gmres(Ab, Lo, Uo, b, precond=2, maxit=3000)
            x64, _, _, _, st64 = orc.gmres(Ab, Lo, Uo, b, precond=1, maxit=3000)
            assert stm == 0 and st64 == 0
            assert abs(int(iters[s, c]) - itm) <= 2, (s, c, iters[s, c], itm)
            x = Xn[off:off + A.n, c]
            assert np.max(np.abs(x - x64)) / np.max(np.abs(x64)) < 1e-8, (s, c)
        off += A.n
