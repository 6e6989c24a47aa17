"""Adjoint kernels through the torch.autograd binding: gradients of
||M^-1 b - t||^2 with respect to b and the block values, for the ISAI apply
(transposed SpMV + masked outer product) and the exact BILU(0) solve
(transposed sync-free SpTRSV over the BCSC view).  Checked against a dense
FP64 reference gradient (small system, 1e-10 relative) and against central
finite differences with h = 1e-6 on 64 random entries of the 256x256
log-normal diffusion system (5e-5 relative to the gradient scale)."""
import numpy as np
import pytest

from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def dense_parts(A, LU):
    M = gen.BSRMatrix(A.nb, A.bs, A.rowptr, A.colind, LU).to_dense()
    return np.tril(M, -1) + np.eye(A.n), np.triu(M)


def block_of(A, dense, p):
    bs = A.bs
    i = np.searchsorted(A.rowptr, p, side="right") - 1
    j = A.colind[p]
    return dense[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs]


def test_ilu_solve_gradient_dense(cuda, orc):
    import torch

    from isai_kernel_gb300.autograd import ilu_solve

    A = gen.lognormal2d(6, bs=4, seed=1)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    b, t = gen.rhs(A.n, 2), gen.rhs(A.n, 3)
    bt = T(b, cuda).requires_grad_(True)
    lut = T(LU, cuda).requires_grad_(True)
    x = ilu_solve(bt, lut, T(A.rowptr, cuda), T(A.colind, cuda), A.nb, A.bs)
    loss = ((x - T(t, cuda)) ** 2).sum()
    loss.backward()
    L, U = dense_parts(A, LU)
    xd = np.linalg.solve(U, np.linalg.solve(L, b))
    yd = np.linalg.solve(L, b)
    gx = 2 * (xd - t)
    lam = np.linalg.solve(U.T, gx)
    mu = np.linalg.solve(L.T, lam)
    np.testing.assert_allclose(bt.grad.cpu().numpy(), mu, rtol=1e-10, atol=1e-12)
    GU, GL = -np.outer(lam, xd), -np.outer(mu, yd)
    g = lut.grad.cpu().numpy()
    for p in range(A.nnzb):
        i = np.searchsorted(A.rowptr, p, side="right") - 1
        j = A.colind[p]
        gu, gl = block_of(A, GU, p), block_of(A, GL, p)
        if j < i:
            want = gl
        elif j > i:
            want = gu
        else:
            want = np.where(np.tril(np.ones((A.bs, A.bs)), -1) > 0, gl, gu)
        np.testing.assert_allclose(g[p], want, rtol=1e-9, atol=1e-11)


def test_isai_apply_gradient_dense(cuda, orc):
    from isai_kernel_gb300.autograd import isai_apply

    A = gen.lognormal2d(6, bs=4, seed=4)
    S = orc.isai_setup(A)
    b, t = gen.rhs(A.n, 5), gen.rhs(A.n, 6)
    bt = T(b, cuda).requires_grad_(True)
    Lv = T(S["McsrL"], cuda).requires_grad_(True)
    Uv = T(S["McsrU"], cuda).requires_grad_(True)
    Lp = (T(S["TrowL"], cuda), T(S["TcolL"], cuda))
    Up = (T(S["TrowU"], cuda), T(S["TcolU"], cuda))
    x = isai_apply(bt, Lv, Uv, Lp, Up, A.nb, A.bs)
    ((x - T(t, cuda)) ** 2).sum().backward()
    ML = gen.BSRMatrix(A.nb, A.bs, S["TrowL"], S["TcolL"], S["McsrL"]).to_dense()
    MU = gen.BSRMatrix(A.nb, A.bs, S["TrowU"], S["TcolU"], S["McsrU"]).to_dense()
    y = ML @ b
    xd = MU @ y
    gx = 2 * (xd - t)
    np.testing.assert_allclose(bt.grad.cpu().numpy(), ML.T @ (MU.T @ gx), rtol=1e-11, atol=1e-12)
    GU, GL = np.outer(gx, y), np.outer(MU.T @ gx, b)
    AU = gen.BSRMatrix(A.nb, A.bs, S["TrowU"], S["TcolU"], S["McsrU"])
    AL = gen.BSRMatrix(A.nb, A.bs, S["TrowL"], S["TcolL"], S["McsrL"])
    gu, gl = Uv.grad.cpu().numpy(), Lv.grad.cpu().numpy()
    for p in range(AU.nnzb):
        np.testing.assert_allclose(gu[p], block_of(AU, GU, p), rtol=1e-11, atol=1e-12)
    for p in range(AL.nnzb):
        np.testing.assert_allclose(gl[p], block_of(AL, GL, p), rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("which", ["ilu", "isai"])
def test_c5_finite_differences(cuda, orc, which):
    """256x256 log-normal diffusion (sigma 1, correlation length 16), loss
    ||M^-1 b - t||^2, central differences h = 1e-6 on 64 random entries of b
    and 64 of the block values."""
    import torch

    from isai_kernel_gb300 import api
    from isai_kernel_gb300.autograd import ilu_solve, isai_apply

    A = gen.lognormal2d(256, bs=4, seed=0)
    rng = np.random.default_rng(0)
    b, t = gen.rhs(A.n, 1), gen.rhs(A.n, 2)
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    P = api.Preconditioner(A.nb, A.bs, row, col, T(A.val, cuda), fp32=False)
    lu, Lf, Uf = P.factors()
    P.close()
    lu = lu.contiguous()
    tt = T(t, cuda)
    if which == "ilu":
        vals = lu
        f = lambda bb, vv: ilu_solve(bb, vv, row, col, A.nb, A.bs)
    else:
        vals = Lf[2].contiguous()
        f = lambda bb, vv: isai_apply(bb, vv, Uf[2], (Lf[0], Lf[1]), (Uf[0], Uf[1]), A.nb, A.bs)
    loss_of = lambda bb, vv: float(((f(bb, vv) - tt) ** 2).sum())
    bt = T(b, cuda).requires_grad_(True)
    vt = vals.clone().requires_grad_(True)
    ((f(bt, vt) - tt) ** 2).sum().backward()
    gb, gv = bt.grad.double(), vt.grad.double()
    h = 1e-6
    bi = rng.choice(A.n, 64, replace=False)
    vi = rng.choice(vals.numel(), 64, replace=False)
    scale_b = float(gb.abs().max())
    scale_v = float(gv.abs().max())
    base_b, base_v = T(b, cuda), vals.clone()
    for i in bi:
        bp, bm = base_b.clone(), base_b.clone()
        bp[i] += h
        bm[i] -= h
        fd = (loss_of(bp, base_v) - loss_of(bm, base_v)) / (2 * h)
        assert abs(fd - float(gb[i])) <= 5e-5 * scale_b, (i, fd, float(gb[i]))
    flat = base_v.view(-1)
    for i in vi:
        vp, vm = base_v.clone(), base_v.clone()
        vp.view(-1)[i] += h
        vm.view(-1)[i] -= h
        fd = (loss_of(base_b, vp) - loss_of(base_b, vm)) / (2 * h)
        assert abs(fd - float(gv.view(-1)[i])) <= 5e-5 * scale_v, (i, fd, float(gv.view(-1)[i]))
    assert flat.numel() == vals.numel()
