"""Oracle properties that need no reference output: the block BILU(0) equals
scalar ILU(0) on the block pattern, L*U = A on the pattern, the ISAI
definition holds on each column pattern, the triangular solves invert the
factors, GMRES converges and counts iterations deterministically."""
import numpy as np
import pytest

from isai_kernel_gb300 import gen


def factor_dense(A, LU):
    M = gen.BSRMatrix(A.nb, A.bs, A.rowptr, A.colind, LU).to_dense()
    n = A.n
    return np.tril(M, -1) + np.eye(n), np.triu(M)


@pytest.mark.parametrize("mk", [lambda: gen.laplace2d(8, bs=4, seed=0),
                                lambda: gen.convdiff3d(4, bs=4, seed=1),
                                lambda: gen.powerlaw(60, bs=8, seed=2, kmax=12),
                                lambda: gen.laplace2d(6, bs=5, seed=3)])
def test_bilu0_is_scalar_ilu0(orc, mk):
    A = mk()
    LU, zp = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    assert zp == -1
    rp, ci, v = A.to_csr()
    sv, zs = orc.csr_ilu0(A.n, rp, ci, v)
    _, _, luv = orc.bsr_to_csr(A.nb, A.bs, A.rowptr, A.colind, LU)
    assert np.array_equal(luv, sv)  # same operations in the same order
    L, U = factor_dense(A, LU)
    D = A.to_dense()
    P = gen.BSRMatrix(A.nb, A.bs, A.rowptr, A.colind, np.ones_like(A.val)).to_dense() != 0
    assert np.max(np.abs((L @ U - D)[P])) < 1e-12 * np.max(np.abs(D))


@pytest.mark.parametrize("level", [1, 2, 3])
def test_isai_definition_and_solves(orc, level):
    """(L M_L)(S_j, j) = e_j and (U M_U)(S_j, j) = e_j on every column pattern
    S_j, for ISAI(1) (A's pattern, as the reference) and ISAI(k) (the
    pattern of A^k)."""
    A = gen.convdiff3d(5, bs=4, seed=0)
    S = orc.isai_setup(A, level=level)
    L, U = factor_dense(A, S["LU"])
    ML = gen.BSRMatrix(A.nb, A.bs, S["TrowL"], S["TcolL"], S["McsrL"]).to_dense()
    MU = gen.BSRMatrix(A.nb, A.bs, S["TrowU"], S["TcolU"], S["McsrU"]).to_dense()
    pat = lambda T: gen.BSRMatrix(A.nb, A.bs, T[0], T[1], np.ones((len(T[1]), A.bs, A.bs))).to_dense() != 0
    PL, PU = pat((S["TrowL"], S["TcolL"])), pat((S["TrowU"], S["TcolU"]))
    I = np.eye(A.n)
    assert np.max(np.abs((L @ ML - I)[PL])) < 1e-12
    assert np.max(np.abs((U @ MU - I)[PU])) < 1e-12
    b = gen.rhs(A.n, 0)
    y = orc.sptrsv_lower(A.nb, A.bs, A.rowptr, A.colind, S["LU"], b)
    x = orc.sptrsv_upper(A.nb, A.bs, A.rowptr, A.colind, S["LU"], y)
    np.testing.assert_allclose(L @ (U @ x), b, rtol=0, atol=1e-12)


def test_pattern_power_and_isai_levels(orc):
    """pattern(A^k) equals the boolean matrix power; denser ISAI levels take
    fewer GMRES iterations on a 3D convection-diffusion system."""
    A = gen.convdiff3d(6, bs=4, seed=0)
    B = np.zeros((A.nb, A.nb), np.int64)
    for i in range(A.nb):
        B[i, A.colind[A.rowptr[i]:A.rowptr[i + 1]]] = 1
    Bk = np.eye(A.nb, dtype=np.int64)
    b = gen.rhs(A.n, 0)
    its = []
    for k in (1, 2, 3):
        Bk = (Bk @ B > 0).astype(np.int64)
        pr, pc = orc.pattern_power(A.nb, A.rowptr, A.colind, k)
        P = np.zeros_like(B)
        for i in range(A.nb):
            row = pc[pr[i]:pr[i + 1]]
            assert np.all(np.diff(row) > 0)
            P[i, row] = 1
        assert np.array_equal(P, Bk)
        S = orc.isai_setup(A, level=k)
        _, it, rr, _, st = orc.gmres((A.rowptr, A.colind, A.val),
                                     (S["TrowL"], S["TcolL"], S["McsrL"]),
                                     (S["TrowU"], S["TcolU"], S["McsrU"]), b, precond=1)
        assert st == 0 and rr <= 1e-10
        its.append(it)
    assert its[0] > its[1] > its[2]


def test_pairs_for_stencils(orc):
    """7-point stencil: one pair per off-diagonal ISAI entry, columns <= 4."""
    A = gen.convdiff3d(6, bs=4, seed=0)
    mp, mi = orc.isai_pattern(A.nb, A.rowptr, A.colind, True)
    pp, pl, ps = orc.pairs_lower(A.nb, A.rowptr, A.colind, mp, mi)
    assert pp[-1] == mp[-1] - A.nb
    assert np.diff(mp).max() == 4


def test_gmres_c1_iterations_deterministic(orc):
    A = gen.laplace2d(16, bs=4, seed=0)
    S = orc.isai_setup(A)
    b = gen.rhs(A.n, 0)
    Ab = (A.rowptr, A.colind, A.val)
    L = (S["TrowL"], S["TcolL"], S["McsrL"])
    U = (S["TrowU"], S["TcolU"], S["McsrU"])
    x, it, rr, hist, st = orc.gmres(Ab, L, U, b, precond=1, maxit=2000)
    assert st == 0 and rr <= 1e-10
    r = b - A.to_dense() @ x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.01e-10
    cores = orc.num_threads()
    orc.set_threads(1)
    x1, it1, rr1, _, _ = orc.gmres(Ab, L, U, b, precond=1, maxit=2000)
    orc.set_threads(cores)
    assert it1 == it and np.array_equal(x1, x)  # chunked reductions: thread-count independent
    x2, it2, rr2, _, st2 = orc.gmres(Ab, L, U, b, precond=2, maxit=2000)
    assert st2 == 0 and abs(it2 - it) <= 2


def test_gmres_nested_oracle(orc):
    """The nested (GMRES-IR) mode: FP64 outer FGMRES(30) over k-step FP32
    inner GMRES solves.  It reaches the FP64 true residual 1e-10, its x is
    within 1e-8 of the FP64 GMRES solution, it is thread-count independent,
    and on the 64 x 64 Laplacian it needs far fewer inner steps in total than
    restarted GMRES(30) needs iterations (1111): the outer space keeps what
    each restart of the flat solver throws away."""
    A = gen.laplace2d(64, bs=4, seed=0)
    S = orc.isai_setup(A)
    b = gen.rhs(A.n, 0)
    Ab = (A.rowptr, A.colind, A.val)
    L = (S["TrowL"], S["TcolL"], S["McsrL"])
    U = (S["TrowU"], S["TcolU"], S["McsrU"])
    x64, it64, _, _, st64 = orc.gmres(Ab, L, U, b, precond=1, maxit=3000)
    assert st64 == 0 and it64 == 1111
    x, it, inner, rr, hist, st = orc.gmres_nested(Ab, L, U, b, inner=20, maxit=300)
    assert st == 0 and rr <= 1e-10 and inner == 20 * it and inner < it64 / 2
    r = b - orc.bcsr_spmv(A.nb, A.bs, A.rowptr, A.colind, A.val, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.01e-10
    assert np.max(np.abs(x - x64)) / np.max(np.abs(x64)) < 1e-8
    cores = orc.num_threads()
    orc.set_threads(1)
    x1, it1, inner1, _, _, _ = orc.gmres_nested(Ab, L, U, b, inner=20, maxit=300)
    orc.set_threads(cores)
    assert it1 == it and inner1 == inner and np.array_equal(x1, x)


def test_dinv_singular_retry(orc):
    """A zero diagonal block: DinvL reads it as unit lower (identity); DinvU
    retries with 1e-12 on the diagonal (isai_bsr.h:114-120, :148-152)."""
    row = np.array([0, 1, 2], np.int32)
    col = np.array([0, 1], np.int32)
    val = np.zeros((2, 4, 4))
    val[0] = np.eye(4) * 2.0
    DL = orc.dinv(2, 4, row, col, val, True)
    DU = orc.dinv(2, 4, row, col, val, False)
    assert np.array_equal(DL[1], np.eye(4))
    np.testing.assert_allclose(DU[1], np.eye(4) * 1e12)
    np.testing.assert_allclose(DU[0], np.eye(4) * 0.5)
