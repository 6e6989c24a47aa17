"""torch.autograd bindings of the preconditioner (test binding for the
adjoint kernels).

* ``IsaiApply``: x = M_U (M_L b).  Backward uses the transposed BSR SpMV for
  the gradient in b and the masked outer product for the block values:
  dL/dM_U = gx y^T, dL/dM_L = (M_U^T gx) b^T on the stored blocks.
* ``IluSolve``: x = U^-1 L^-1 b on the packed BILU(0) factor.  Backward uses
  the transposed sync-free solves over the BCSC view: lam = U^-T gx,
  mu = L^-T lam; dL/db = mu, dL/dU = -lam x^T, dL/dL = -mu y^T (each on its
  triangle of the packed factor).

Every product runs in libbilu_isai.so through the C ABI.
"""
from __future__ import annotations

import torch

from . import api


class IsaiApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, b, Lval, Uval, Lrow, Lcol, Urow, Ucol, nb: int, bs: int):
        y = api.bcsr_spmv(nb, bs, Lrow, Lcol, Lval.detach(), b.detach())
        x = api.bcsr_spmv(nb, bs, Urow, Ucol, Uval.detach(), y)
        ctx.save_for_backward(b.detach(), y, Lval, Uval, Lrow, Lcol, Urow, Ucol)
        ctx.nb, ctx.bs = nb, bs
        return x

    @staticmethod
    def backward(ctx, gx):
        b, y, Lval, Uval, Lrow, Lcol, Urow, Ucol = ctx.saved_tensors
        nb, bs = ctx.nb, ctx.bs
        gx = gx.contiguous()
        gy = api.bcsr_spmv_transpose(nb, bs, Urow, Ucol, Uval.detach(), gx)
        gb = api.bcsr_spmv_transpose(nb, bs, Lrow, Lcol, Lval.detach(), gy)
        gU = api.masked_outer(nb, bs, Urow, Ucol, gx, y) if ctx.needs_input_grad[2] else None
        gL = api.masked_outer(nb, bs, Lrow, Lcol, gy, b) if ctx.needs_input_grad[1] else None
        return gb, gL, gU, None, None, None, None, None, None


def lower_mask(nb: int, bs: int, row, col):
    """Per-element mask of the L part of a packed factor: strictly lower
    blocks, and the strict lower triangle of diagonal blocks."""
    rows = torch.repeat_interleave(torch.arange(nb, device=row.device, dtype=torch.int32),
                                   (row[1:] - row[:-1]).long())
    c = col.long()
    r = rows.long()
    blk_lower = (c < r).view(-1, 1, 1)
    blk_diag = (c == r).view(-1, 1, 1)
    tri = torch.tril(torch.ones(bs, bs, dtype=torch.bool, device=row.device), -1)
    return blk_lower | (blk_diag & tri)


class IluSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, b, LU, row, col, nb: int, bs: int):
        y = api.sptrsv(nb, bs, row, col, LU.detach(), b.detach(), lower=True)
        x = api.sptrsv(nb, bs, row, col, LU.detach(), y, lower=False)
        ctx.save_for_backward(LU, row, col, y, x)
        ctx.nb, ctx.bs = nb, bs
        return x

    @staticmethod
    def backward(ctx, gx):
        LU, row, col, y, x = ctx.saved_tensors
        nb, bs = ctx.nb, ctx.bs
        lam = api.sptrsv(nb, bs, row, col, LU.detach(), gx.contiguous(), lower=False,
                         transpose=True)
        mu = api.sptrsv(nb, bs, row, col, LU.detach(), lam, lower=True, transpose=True)
        gLU = None
        if ctx.needs_input_grad[1]:
            gU = api.masked_outer(nb, bs, row, col, lam, x, scale=-1.0)
            gL = api.masked_outer(nb, bs, row, col, mu, y, scale=-1.0)
            gLU = torch.where(lower_mask(nb, bs, row, col), gL, gU)
        return mu, gLU, None, None, None, None


def isai_apply(b, Lval, Uval, L, U, nb: int, bs: int):
    """Differentiable x = M_U (M_L b); L, U are (rowptr, colind) of the BCSR
    factors, Lval/Uval their block values."""
    return IsaiApply.apply(b, Lval, Uval, L[0], L[1], U[0], U[1], nb, bs)


def ilu_solve(b, LU, row, col, nb: int, bs: int):
    """Differentiable x = U^-1 L^-1 b on the packed BILU(0) factor."""
    return IluSolve.apply(b, LU, row, col, nb, bs)
