"""GPU parity: every CUDA entry point, called through the C ABI
(libbilu_isai.so via ctypes), against the CPU oracle and the golden vectors
of the reference's own host code.

Tolerances: integer / index / pattern / copy outputs bit-exact; FP64 factors,
inverses, ISAI values and triangular solves within 1e-12 relative (max abs
difference over max abs value); FP64 SpMV within 1e-13 relative; FP32-stored
SpMV within 2e-6 relative of the FP32 oracle; FP64 GMRES takes exactly the
oracle's iteration count."""
import numpy as np
import pytest

from conftest import golden
from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu

MATS = ["laplace2d_s12", "convdiff3d_s5", "powerlaw_nb120", "laplace2d_s9_bs5"]


def T(a, dev):
    import torch

    a = np.ascontiguousarray(a)
    return torch.from_numpy(a).to(dev)


def N(t):
    return t.detach().cpu().numpy()


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if b.size else 0.0


def mats():
    return {
        "c1_s16": gen.laplace2d(16, bs=4, seed=0),
        "c2_s6": gen.convdiff3d(6, bs=4, seed=0),
        "c3_nb200": gen.powerlaw(200, bs=8, seed=0, kmax=30),
        "bs5_s7": gen.laplace2d(7, bs=5, seed=2),
    }


# ------------------------------------------------------------------ formats
@pytest.mark.parametrize("bs", [4, 5, 8])
def test_csr_to_bsr_golden(cuda, bs):
    from isai_kernel_gb300 import api

    g = golden(f"c2b_bs{bs}")
    nb, r, c, v = api.csr_to_bsr5(int(g["n"]), bs, T(g["csr_row"], cuda), T(g["csr_col"], cuda),
                                  T(g["csr_val"], cuda))
    assert np.array_equal(N(r), g["bsr_row"]) and np.array_equal(N(c), g["bsr_col"])
    assert np.array_equal(N(v), g["bsr_val"])


@pytest.mark.parametrize("name", MATS)
def test_patterns_map_golden(cuda, name):
    from isai_kernel_gb300 import api

    g = golden(name)
    nb = int(g["nb"])
    row, col = T(g["row"], cuda), T(g["col"], cuda)
    for lower, tag in ((True, "L"), (False, "U")):
        mp, mi = api.build_bcsc_pattern_from_bsr_scalarILU(nb, row, col, lower)
        assert np.array_equal(N(mp), g[f"Mptr{tag}"]) and np.array_equal(N(mi), g[f"Mind{tag}"])
        tr, tc = api.build_triangular_bcsr_pattern_from_A(nb, row, col, lower)
        assert np.array_equal(N(tr), g[f"Trow{tag}"]) and np.array_equal(N(tc), g[f"Tcol{tag}"])
        m = api.build_map_bcsc2bcsr_host(nb, mp, mi, tr, tc)
        assert np.array_equal(N(m), g[f"map{tag}"])


@pytest.mark.parametrize("name", MATS)
def test_spmv_reorder_bcsc_golden(cuda, name):
    from isai_kernel_gb300 import api

    g = golden(name)
    nb, bs = int(g["nb"]), int(g["bs"])
    y = api.bcsr_spmv(nb, bs, T(g["row"], cuda), T(g["col"], cuda), T(g["val"], cuda),
                      T(g["x"], cuda))
    assert relerr(N(y), g["spmv_y"]) < 1e-13
    vals = api.reorder_bcsc_val_to_bcsr(T(g["mapL"], cuda), T(g["bcsc_val"], cuda))
    yb = api.bcsr_spmv(nb, bs, T(g["TrowL"], cuda), T(g["TcolL"], cuda), vals, T(g["x"], cuda))
    assert relerr(N(yb), g["bcsc_y"]) < 1e-13
    rp, ci, v = api.bcsc_to_bcsr(nb, nb, bs, T(g["MptrL"], cuda), T(g["MindL"], cuda),
                                 T(g["bcsc_val"], cuda))
    assert np.array_equal(N(rp), g["TrowL"]) and np.array_equal(N(ci), g["TcolL"])
    assert np.array_equal(N(v), N(vals))


@pytest.mark.parametrize("name", list(mats()))
def test_bsr2csr_and_back(cuda, orc, name):
    from isai_kernel_gb300 import api

    A = mats()[name]
    rp, ci, v = api.bsr2csr(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda))
    orp, oci, ov = orc.bsr_to_csr(A.nb, A.bs, A.rowptr, A.colind, A.val)
    assert np.array_equal(N(rp), orp) and np.array_equal(N(ci), oci) and np.array_equal(N(v), ov)
    nb, r2, c2, v2 = api.csr_to_bsr5(A.n, A.bs, rp, ci, v)
    assert np.array_equal(N(r2), A.rowptr) and np.array_equal(N(c2), A.colind)
    assert np.array_equal(N(v2), A.val)


def test_transpose_view(cuda):
    from isai_kernel_gb300 import api

    A = gen.powerlaw(150, bs=8, seed=5, kmax=25)
    tr, tc, tv = api.bsr_transpose(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda))
    At = gen.BSRMatrix(A.nb, A.bs, N(tr), N(tc), N(tv))
    assert np.array_equal(At.to_dense(), A.to_dense().T)


# ------------------------------------------------------------------ factor + ISAI
@pytest.mark.parametrize("name", list(mats()))
def test_bilu0_matches_oracle(cuda, orc, name):
    from isai_kernel_gb300 import api

    A = mats()[name]
    ref, zp = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    v = T(A.val, cuda).clone()
    info = api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), v)
    assert info == zp == -1
    assert relerr(N(v), ref) < 1e-12


@pytest.mark.parametrize("name", list(mats()))
def test_isai_setup_matches_oracle(cuda, orc, name):
    """Dinv, pair lists and ISAI-L/U values on the oracle's factor."""
    from isai_kernel_gb300 import api

    A = mats()[name]
    S = orc.isai_setup(A)
    row, col, LU = T(A.rowptr, cuda), T(A.colind, cuda), T(S["LU"], cuda)
    for lower, tag in ((True, "L"), (False, "U")):
        D = api.build_Dinv(A.nb, A.bs, row, col, LU, lower)
        assert relerr(N(D), S[f"Dinv{tag}"]) < 1e-12
        mp, mi = T(S[f"Mptr{tag}"], cuda), T(S[f"Mind{tag}"], cuda)
        pp, pl, ps, nmax = api.build_pairs(A.nb, row, col, mp, mi, lower)
        assert nmax == int(np.diff(S[f"Mptr{tag}"]).max())
        if lower:
            assert np.array_equal(N(pp), S["PairPtr"])
            assert np.array_equal(N(pl), S["PairPLocal"]) and np.array_equal(N(ps), S["PairSrc"])
        M = api.isai_compute(A.nb, A.bs, LU, mp, mi, pp, pl, ps, D, lower)
        assert relerr(N(M), S[f"Mcsc{tag}"]) < 1e-12


def test_upper_pairs_definition(cuda, orc):
    """M_U pair list: for entry idx of column j, every p > idx (descending)
    whose block U(t, S_j[p]) is stored, with its BSR position."""
    from isai_kernel_gb300 import api

    A = gen.powerlaw(90, bs=8, seed=3, kmax=20)
    mp, mi = orc.isai_pattern(A.nb, A.rowptr, A.colind, False)
    pp, pl, ps, _ = api.build_pairs(A.nb, T(A.rowptr, cuda), T(A.colind, cuda), T(mp, cuda),
                                    T(mi, cuda), False)
    pp, pl, ps = N(pp), N(pl), N(ps)
    for j in range(A.nb):
        s, e = mp[j], mp[j + 1]
        for idx in range(e - s):
            t = mi[s + idx]
            want = []
            for p in range(e - s - 1, idx, -1):
                hit = np.nonzero(A.colind[A.rowptr[t]:A.rowptr[t + 1]] == mi[s + p])[0]
                if hit.size:
                    want.append((p, A.rowptr[t] + hit[0]))
            got = list(zip(pl[pp[s + idx]:pp[s + idx + 1]], ps[pp[s + idx]:pp[s + idx + 1]]))
            assert got == want


# ------------------------------------------------------------------ apply
@pytest.mark.parametrize("name", list(mats()))
def test_spmv_fp64_fp32(cuda, orc, name):
    import torch
    from isai_kernel_gb300 import api

    A = mats()[name]
    x = gen.rhs(A.n, 11)
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    y = api.bcsr_spmv(A.nb, A.bs, row, col, T(A.val, cuda), T(x, cuda))
    assert relerr(N(y), orc.bcsr_spmv(A.nb, A.bs, A.rowptr, A.colind, A.val, x)) < 1e-13
    v32 = A.val.astype(np.float32)
    y32 = orc.bcsr_spmv_f32(A.nb, A.bs, A.rowptr, A.colind, v32, x.astype(np.float32))
    for xt, yt in ((torch.float32, torch.float32), (torch.float64, torch.float64),
                   (torch.float32, torch.float64), (torch.float64, torch.float32)):
        xin = T(x, cuda).to(xt)
        out = torch.empty(A.n, dtype=yt, device=cuda)
        api.bcsr_spmv(A.nb, A.bs, row, col, T(v32, cuda), xin, out)
        ref = y32 if xt == torch.float32 else orc.bcsr_spmv_f32(
            A.nb, A.bs, A.rowptr, A.colind, v32, x.astype(np.float32))
        assert relerr(N(out), ref) < 2e-6


@pytest.mark.parametrize("k", [1, 8, 32, 40])
def test_spmm_matches_spmv_columns(cuda, orc, k):
    from isai_kernel_gb300 import api

    A = gen.laplace2d(12, bs=4, seed=1)
    X = gen.rhs(A.n, 4, k=k) if k > 1 else gen.rhs(A.n, 4).reshape(-1, 1)
    row, col, val = T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda)
    Y = N(api.bcsr_spmm(A.nb, A.bs, row, col, val, T(X, cuda)))
    for c in range(k):
        ref = orc.bcsr_spmv(A.nb, A.bs, A.rowptr, A.colind, A.val, np.ascontiguousarray(X[:, c]))
        assert relerr(Y[:, c], ref) < 1e-13
    Y32 = N(api.bcsr_spmm(A.nb, A.bs, row, col, val.float(), T(X, cuda)))
    ref32 = orc.bcsr_spmv_f32(A.nb, A.bs, A.rowptr, A.colind, A.val.astype(np.float32),
                              np.ascontiguousarray(X[:, 0]).astype(np.float32))
    assert relerr(Y32[:, 0], ref32) < 1e-5


def test_spmv_transpose_and_outer(cuda):
    from isai_kernel_gb300 import api

    A = gen.powerlaw(100, bs=8, seed=9, kmax=20)
    D = A.to_dense()
    x, u = gen.rhs(A.n, 1), gen.rhs(A.n, 2)
    row, col, val = T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda)
    y = N(api.bcsr_spmv_transpose(A.nb, A.bs, row, col, val, T(x, cuda)))
    assert relerr(y, D.T @ x) < 1e-13
    G = N(api.masked_outer(A.nb, A.bs, row, col, T(u, cuda), T(x, cuda), 2.0))
    bs = A.bs
    for p in range(0, A.nnzb, 7):
        i = np.searchsorted(A.rowptr, p, side="right") - 1
        j = A.colind[p]
        want = 2.0 * np.outer(u[i * bs:(i + 1) * bs], x[j * bs:(j + 1) * bs])
        assert np.allclose(G[p], want, rtol=1e-15, atol=0)


# ------------------------------------------------------------------ sync-free solves
@pytest.mark.parametrize("name", list(mats()))
def test_sptrsv_matches_oracle(cuda, orc, name):
    from isai_kernel_gb300 import api

    A = mats()[name]
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    b = gen.rhs(A.n, 3)
    row, col, lu = T(A.rowptr, cuda), T(A.colind, cuda), T(LU, cuda)
    y = api.sptrsv(A.nb, A.bs, row, col, lu, T(b, cuda), lower=True)
    yo = orc.sptrsv_lower(A.nb, A.bs, A.rowptr, A.colind, LU, b)
    assert relerr(N(y), yo) < 1e-12
    x = api.sptrsv(A.nb, A.bs, row, col, lu, y, lower=False)
    xo = orc.sptrsv_upper(A.nb, A.bs, A.rowptr, A.colind, LU, yo)
    assert relerr(N(x), xo) < 1e-12


def test_sptrsv_transposed(cuda, orc):
    from isai_kernel_gb300 import api

    A = gen.powerlaw(120, bs=8, seed=4, kmax=20)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    M = gen.BSRMatrix(A.nb, A.bs, A.rowptr, A.colind, LU).to_dense()
    L, U = np.tril(M, -1) + np.eye(A.n), np.triu(M)
    b = gen.rhs(A.n, 6)
    row, col, lu = T(A.rowptr, cuda), T(A.colind, cuda), T(LU, cuda)
    xl = N(api.sptrsv(A.nb, A.bs, row, col, lu, T(b, cuda), lower=True, transpose=True))
    xu = N(api.sptrsv(A.nb, A.bs, row, col, lu, T(b, cuda), lower=False, transpose=True))
    assert relerr(xl, np.linalg.solve(L.T, b)) < 1e-10
    assert relerr(xu, np.linalg.solve(U.T, b)) < 1e-10


@pytest.mark.parametrize("name", ["laplace2d_s12", "convdiff3d_s5", "powerlaw_nb120"])
def test_sptrsv_level_and_syncfree_schedules(cuda, orc, name):
    """Analysis once, then the level-scheduled and the sync-free solve on
    it: identical x (each row's arithmetic does not depend on the schedule),
    equal to the oracle within 1e-12; level counts match the oracle's
    longest-path levels."""
    import torch

    from isai_kernel_gb300 import _lib, api

    d = golden(name)
    nb, bs = int(d["nb"]), int(d["bs"])
    LU, _ = orc.bsrilu0(nb, bs, d["row"], d["col"], d["val"])
    row, col, lu = T(d["row"], cuda), T(d["col"], cuda), T(LU, cuda)
    nnzb = int(d["col"].shape[0])
    b = gen.rhs(nb * bs, 5)
    L = _lib.lib()
    for lower in (1, 0):
        info = api._ws(L.bilu_sptrsv_analysis_bytes(nb), cuda)
        ws = api._ws(max(L.bilu_sptrsv_analysis_ws_bytes(nb, nnzb), L.bilu_sptrsv_solve_ws_bytes(nb)),
                     cuda)
        api.call("bilu_sptrsv_analysis", nb, nnzb, bs, api._p(row), api._p(col), lower,
                 api._p(info), api._p(ws), ws.numel(), api._s())
        bd = T(b, cuda)
        x1, x2, x3 = torch.empty_like(bd), torch.empty_like(bd), torch.empty_like(bd)
        for fn, x in (("bilu_sptrsv_solve_level", x1), ("bilu_sptrsv_solve_syncfree", x2),
                      ("bilu_sptrsv_solve", x3)):
            api.call(fn, nb, bs, api._p(row), api._p(col), api._p(lu), lower, lower, api._p(info),
                     api._p(bd), api._p(x), api._p(ws), ws.numel(), api._s())
        assert torch.equal(x1, x2) and torch.equal(x1, x3)
        ref = (orc.sptrsv_lower if lower else orc.sptrsv_upper)(nb, bs, d["row"], d["col"],
                                                                LU, b)
        assert relerr(N(x1), ref) < 1e-12
        # level sizes: oracle longest-path levels over the same DAG
        lv = np.zeros(nb, np.int64)
        rp, ci = d["row"], d["col"]
        rows = range(nb) if lower else range(nb - 1, -1, -1)
        for i in rows:
            deps = ci[rp[i]:rp[i + 1]]
            deps = deps[deps < i] if lower else deps[deps > i]
            lv[i] = 1 + (lv[deps].max() if deps.size else 0)
        words = N(info).view(np.int32)
        # record layout: diag | order | lvl_ptr | nlev, each carved on 256 B
        def carve(n):
            return ((n * 4 + 255) // 256) * 64
        o_lvl = 2 * carve(nb + 1)
        o_nlev = o_lvl + carve(nb + 2)
        nlev = int(words[o_nlev])
        ptr = words[o_lvl:o_lvl + nlev + 1]
        assert nlev == lv.max() and ptr[-1] == nb
        assert np.array_equal(np.diff(ptr), np.bincount(lv - 1, minlength=nlev))


@pytest.mark.parametrize("bs,side", [(4, 7), (5, 6), (8, 5)])
@pytest.mark.parametrize("kind", ["laplace2d", "convdiff3d"])
def test_flow_solve_block_sizes(cuda, orc, kind, bs, side):
    """The level-order (flow) solve at every built block size (16/bs
    dependencies staged in registers: 4 at bs 4, 3 at bs 5, 1 at bs 8, the
    rest read in the row loop): bit-identical to the sync-free solve and
    within 1e-12 of the oracle, both triangles."""
    import torch

    from isai_kernel_gb300 import _lib, api

    A = (gen.laplace2d(side * 2, bs=bs, seed=bs) if kind == "laplace2d"
         else gen.convdiff3d(side, bs=bs, seed=bs))
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col, lu = T(A.rowptr, cuda), T(A.colind, cuda), T(LU, cuda)
    bh = gen.rhs(A.n, bs)
    b = T(bh, cuda)
    L = _lib.lib()
    for lower in (1, 0):
        info = api._ws(L.bilu_sptrsv_analysis_bytes(A.nb), cuda)
        ws = api._ws(max(L.bilu_sptrsv_analysis_ws_bytes(A.nb, A.nnzb),
                         L.bilu_sptrsv_solve_ws_bytes(A.nb)), cuda)
        api.call("bilu_sptrsv_analysis", A.nb, A.nnzb, bs, api._p(row), api._p(col), lower,
                 api._p(info), api._p(ws), ws.numel(), api._s())
        xs = []
        for fn in ("bilu_sptrsv_solve_level", "bilu_sptrsv_solve_syncfree"):
            x = torch.empty_like(b)
            api.call(fn, A.nb, bs, api._p(row), api._p(col), api._p(lu), lower, lower,
                     api._p(info), api._p(b), api._p(x), api._p(ws), ws.numel(), api._s())
            xs.append(N(x))
        assert np.array_equal(xs[0], xs[1])
        ref = (orc.sptrsv_lower if lower else orc.sptrsv_upper)(A.nb, bs, A.rowptr, A.colind,
                                                                 LU, bh)
        assert relerr(xs[0], ref) < 1e-12


@pytest.mark.parametrize("name", ["c1_s16", "c2_s6", "c3_nb200", "bs5_s7", "long_rows"])
def test_bilu0_both_schedules(cuda, orc, name):
    """BILU(0) under the level schedule (a bs-lane group per row) and the
    sync-free one (a warp per row, tickets in level order): identical
    factors, within 1e-12 of the oracle."""
    from isai_kernel_gb300 import api

    A = gen.powerlaw(400, bs=8, seed=5, kmax=150) if name == "long_rows" else mats()[name]
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    out = []
    for sched in (0, 1):
        lu = T(A.val, cuda).clone()
        assert api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, row, col, lu, schedule=sched) == -1
        out.append(N(lu))
    assert np.array_equal(out[0], out[1])
    assert relerr(out[0], LU) < 1e-12


def test_bilu0_dense_rows_both_schedules(cuda, orc):
    """A dense 40 x 40 block pattern: the (row, dependency) pairs whose two
    candidate lists both hold more than 32 blocks are counted by a whole
    warp before the sync-free factorisation; identical factors under both
    schedules, within 1e-12 of the oracle."""
    from isai_kernel_gb300 import api

    nb, bs = 40, 4
    rng = np.random.default_rng(17)
    rowptr = (np.arange(nb + 1) * nb).astype(np.int32)
    colind = np.tile(np.arange(nb, dtype=np.int32), nb)
    val = rng.uniform(-1.0, 1.0, (nb * nb, bs, bs))
    for i in range(nb):
        val[i * nb + i] += np.eye(bs) * (4.0 * nb)
    A = gen.BSRMatrix(nb, bs, rowptr, colind, val)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    out = []
    for sched in (0, 1):
        lu = T(A.val, cuda).clone()
        assert api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, row, col, lu, schedule=sched) == -1
        out.append(N(lu))
    assert np.array_equal(out[0], out[1])
    assert relerr(out[0], LU) < 1e-12


@pytest.mark.parametrize("bs", [4, 5, 8])
def test_dinv_retry_blocks(cuda, orc, bs):
    """Diagonal-block inverses with an all-zero block and a 1e-15 pivot:
    the lower inverse reads the unit lower part, the upper one retries with
    1e-12 added to the diagonal (isai_bsr.h:114-120); every block within
    1e-12 of the oracle's Gauss-Jordan."""
    from isai_kernel_gb300 import api

    nb = 6
    rng = np.random.default_rng(4)
    row = np.arange(nb + 1, dtype=np.int32)
    col = np.arange(nb, dtype=np.int32)
    val = rng.uniform(-1.0, 1.0, (nb, bs, bs)) + np.eye(bs) * 3.0
    val[1] = 0.0
    val[2][1, 1] = 1e-15
    for lower in (True, False):
        D = N(api.build_Dinv(nb, bs, T(row, cuda), T(col, cuda), T(val, cuda), lower))
        ref = orc.dinv(nb, bs, row, col, val, lower)
        for k in range(nb):
            assert relerr(D[k], ref[k]) < 1e-12, (lower, k)
    assert abs(ref[1][0, 0] - 1e12) < 1.0  # the upper retry ran (zero block)


@pytest.mark.parametrize("name", ["c2_s6", "c3_nb200"])
def test_exact_ilu_gmres_both_schedules(cuda, orc, name):
    """GMRES with the exact BILU(0) under both schedules of the factor and
    the triangular solves: the same iterations and the same x bit for bit,
    equal to the oracle's iteration count."""
    from isai_kernel_gb300 import api

    A = mats()[name]
    b = T(gen.rhs(A.n, 0), cuda)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    _, ito, _, _, st = orc.gmres((A.rowptr, A.colind, A.val), (A.rowptr, A.colind, LU), None,
                                 N(b), precond=3, maxit=3000)
    assert st == 0
    xs, its = [], []
    for sched in (0, 1):
        p = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda),
                               ilu=True, schedule=sched)
        x, res = p.solve(b, prec=api.BILU_ILU, maxit=3000)
        assert res.converged
        xs.append(N(x))
        its.append(res.iters)
        p.close()
    assert its[0] == its[1] == ito
    assert np.array_equal(xs[0], xs[1])


def test_exact_ilu_only_handle(cuda, orc):
    """A handle set up for the exact ILU apply alone builds no ISAI: the ILU
    solve matches a full handle's bit for bit, and the ISAI modes report
    BILU_ERR_ARG instead of running on missing factors."""
    from isai_kernel_gb300 import api
    from isai_kernel_gb300._lib import BiluError

    A = mats()["c2_s6"]
    b = T(gen.rhs(A.n, 0), cuda)
    args = (A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda))
    full = api.Preconditioner(*args, fp32=True, ilu=True)
    only = api.Preconditioner(*args, fp32=False, ilu=True)
    x1, r1 = full.solve(b, prec=api.BILU_ILU, maxit=3000)
    x2, r2 = only.solve(b, prec=api.BILU_ILU, maxit=3000)
    assert r1.converged and r1.iters == r2.iters and np.array_equal(N(x1), N(x2))
    for prec in (api.BILU_FP64, api.BILU_FP32):
        with pytest.raises(BiluError) as e:
            only.solve(b, prec=prec, maxit=10)
        assert e.value.status == -1
    full.close()
    only.close()


@pytest.mark.parametrize("bs", [4, 5, 8])
def test_spmv_long_rows(cuda, orc, bs):
    """SpMV on a power-law pattern with rows of up to ~150 blocks (rows over
    64 blocks are summed by the whole CTA): FP64 within 1e-12 of the
    oracle's row-order sum, FP32-stored values within FP32 rounding, and the
    result does not depend on whether the row-length check is cached."""
    import torch

    from isai_kernel_gb300 import api

    A = gen.powerlaw(600, bs=bs, seed=9, kmax=150)
    lens = np.diff(A.rowptr)
    assert lens.max() > 64
    x = gen.rhs(A.n, 11)
    # every device buffer stays referenced until the kernels have run
    row, col, val, xd = T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda), T(x, cuda)
    y = torch.empty(A.n, dtype=torch.float64, device="cuda")
    for _ in range(2):  # the second call uses the cached check
        api.call("bilu_bcsr_spmv", A.nb, bs, api._p(row), api._p(col), api._p(val), api._p(xd),
                 api._p(y), api._s())
        ref = orc.bcsr_spmv(A.nb, bs, A.rowptr, A.colind, A.val, x)
        assert relerr(N(y), ref) < 1e-12
    v32 = T(A.val.astype(np.float32), cuda)
    x32 = T(x.astype(np.float32), cuda)
    y32 = torch.empty(A.n, dtype=torch.float32, device="cuda")
    api.call("bilu_bcsr_spmv_f32", A.nb, bs, api._p(row), api._p(col), api._p(v32),
             api._p(x32), 1, api._p(y32), 1, api._s())
    ref32 = orc.bcsr_spmv(A.nb, bs, A.rowptr, A.colind, A.val.astype(np.float32).astype(np.float64),
                          x.astype(np.float32).astype(np.float64))
    assert relerr(N(y32).astype(np.float64), ref32) < 1e-5


@pytest.mark.parametrize("bs", [4, 5, 8])
def test_spmv_every_layout(cuda, orc, bs):
    """Every SpMV layout (with and without the CTA's long-row pass, one or
    two block rows per lane group) on a pattern with rows of up to ~150
    blocks, and the layout the check finds for it and for a stencil: FP64
    within 1e-12 of the oracle and FP32-stored values within 1e-5 of the
    oracle on the rounded values, whichever kernel runs."""
    import ctypes

    import torch

    from isai_kernel_gb300 import api

    A = gen.powerlaw(600, bs=bs, seed=9, kmax=150)
    x = gen.rhs(A.n, 13)
    row, col, val, xd = T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda), T(x, cuda)
    ref = orc.bcsr_spmv(A.nb, bs, A.rowptr, A.colind, A.val, x)
    v32 = A.val.astype(np.float32)
    ref32 = orc.bcsr_spmv(A.nb, bs, A.rowptr, A.colind, v32.astype(np.float64),
                          x.astype(np.float32).astype(np.float64))
    val32, x32 = T(v32, cuda), T(x.astype(np.float32), cuda)
    lay = ctypes.c_int(-1)
    api.call("bilu_spmv_layout", A.nb, bs, api._p(row), api._s(), ctypes.byref(lay))
    assert lay.value == 3  # rows of ~150 blocks, 12 on average
    y = torch.empty(A.n, dtype=torch.float64, device="cuda")
    y32 = torch.empty(A.n, dtype=torch.float32, device="cuda")
    for layout in (0, 1, 2, 3):
        api.call("bilu_debug_spmv_layout_set", A.nb, bs, api._p(row), layout)
        y.fill_(float("nan"))
        api.call("bilu_bcsr_spmv", A.nb, bs, api._p(row), api._p(col), api._p(val), api._p(xd),
                 api._p(y), api._s())
        assert relerr(N(y), ref) < 1e-12, layout
        y32.fill_(float("nan"))
        api.call("bilu_bcsr_spmv_f32", A.nb, bs, api._p(row), api._p(col), api._p(val32),
                 api._p(x32), 1, api._p(y32), 1, api._s())
        assert relerr(N(y32).astype(np.float64), ref32) < 1e-5, layout
    # a 7-point stencil (~6 blocks a row) and a 5-point one (~5): no long rows
    S = gen.convdiff3d(6, bs=4, seed=0) if bs == 4 else gen.laplace2d(7, bs=bs, seed=2)
    srow = T(S.rowptr, cuda)
    api.call("bilu_spmv_layout", S.nb, bs, api._p(srow), api._s(), ctypes.byref(lay))
    assert lay.value == (2 if S.nnzb > 5 * S.nb else 0)


def test_long_rows_take_the_warp_path(cuda, orc):
    """A power-law system with rows of more than 32 dependencies (up to 126
    here): the level kernels switch to a warp per row.  BILU(0) within 1e-12
    of the oracle, level and sync-free solves bit-identical and within 1e-12
    of the oracle's."""
    import torch

    from isai_kernel_gb300 import _lib, api

    A = gen.powerlaw(400, bs=8, seed=5, kmax=150)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    lu = T(A.val, cuda).clone()
    assert api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, row, col, lu) == -1
    assert relerr(N(lu), LU) < 1e-12
    L = _lib.lib()
    b = gen.rhs(A.n, 7)
    bd = T(b, cuda)
    for lower in (1, 0):
        info = api._ws(L.bilu_sptrsv_analysis_bytes(A.nb), cuda)
        ws = api._ws(max(L.bilu_sptrsv_analysis_ws_bytes(A.nb, A.nnzb),
                         L.bilu_sptrsv_solve_ws_bytes(A.nb)), cuda)
        api.call("bilu_sptrsv_analysis", A.nb, A.nnzb, A.bs, api._p(row), api._p(col), lower,
                 api._p(info), api._p(ws), ws.numel(), api._s())
        x1, x2, x3 = torch.empty_like(bd), torch.empty_like(bd), torch.empty_like(bd)
        for fn, x in (("bilu_sptrsv_solve_level", x1), ("bilu_sptrsv_solve_syncfree", x2),
                      ("bilu_sptrsv_solve", x3)):
            api.call(fn, A.nb, A.bs, api._p(row), api._p(col), api._p(lu), lower, lower,
                     api._p(info), api._p(bd), api._p(x), api._p(ws), ws.numel(), api._s())
        assert torch.equal(x1, x2) and torch.equal(x1, x3)
        ref = (orc.sptrsv_lower if lower else orc.sptrsv_upper)(A.nb, A.bs, A.rowptr, A.colind,
                                                                LU, b)
        assert relerr(N(x1), ref) < 1e-12


def test_sptrsv_timeout_path(cuda, orc):
    """A row that never publishes: dependants give up after a short bounded
    wait, the call reports BILU_ERR_TIMEOUT, and the context stays usable."""
    import ctypes

    from isai_kernel_gb300 import _lib, api

    A = gen.laplace2d(10, bs=4, seed=0)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col, lu = T(A.rowptr, cuda), T(A.colind, cuda), T(LU, cuda)
    b = T(gen.rhs(A.n, 3), cuda)
    x = b.clone()
    ws = api._ws(_lib.lib().bilu_sptrsv_ws_bytes(A.nb, A.nnzb), cuda)
    st = _lib.lib().bilu_debug_sptrsv_withhold(
        A.nb, A.bs, api._p(row), api._p(col), api._p(lu), 1, api._p(b), api._p(x), 5,
        ctypes.c_longlong(1 << 14), api._p(ws), ws.numel(), api._s())
    assert st == -4  # BILU_ERR_TIMEOUT
    y = api.sptrsv(A.nb, A.bs, row, col, lu, b, lower=True)
    yo = orc.sptrsv_lower(A.nb, A.bs, A.rowptr, A.colind, LU, N(b))
    assert relerr(N(y), yo) < 1e-12


@pytest.mark.parametrize("lower", [1, 0])
def test_flow_solve_withheld_row_times_out(cuda, orc, lower):
    """The level-order (flow) solve with a row that never stores its x
    entries: the rows reading them give up after a short bounded wait, the
    call reports BILU_ERR_TIMEOUT, and the next solve is correct."""
    import ctypes

    import torch

    from isai_kernel_gb300 import _lib, api

    A = gen.convdiff3d(6, bs=4, seed=1)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col, lu = T(A.rowptr, cuda), T(A.colind, cuda), T(LU, cuda)
    b = T(gen.rhs(A.n, 4), cuda)
    x = torch.empty_like(b)
    L = _lib.lib()
    ws = api._ws(L.bilu_sptrsv_ws_bytes(A.nb, A.nnzb), cuda)
    st = L.bilu_debug_sptrsv_withhold_flow(
        A.nb, A.nnzb, A.bs, api._p(row), api._p(col), api._p(lu), lower, api._p(b), api._p(x),
        A.nb // 3, ctypes.c_longlong(1 << 12), api._p(ws), ws.numel(), api._s())
    assert st == -4  # BILU_ERR_TIMEOUT
    y = api.sptrsv(A.nb, A.bs, row, col, lu, b, lower=bool(lower))
    ref = (orc.sptrsv_lower if lower else orc.sptrsv_upper)(A.nb, A.bs, A.rowptr, A.colind, LU,
                                                             N(b))
    assert relerr(N(y), ref) < 1e-12


def test_nan_in_b_propagates_without_waiting(cuda, orc):
    """A NaN in b is an ordinary value for the flow solve (only the pending
    pattern means "not computed"): the solve finishes, the rows that depend
    on the NaN row are NaN, and the level-order and sync-free solves agree
    entry for entry."""
    import torch

    from isai_kernel_gb300 import _lib, api

    A = gen.convdiff3d(6, bs=4, seed=2)
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col, lu = T(A.rowptr, cuda), T(A.colind, cuda), T(LU, cuda)
    bh = gen.rhs(A.n, 5)
    bh[4 * 20 + 1] = np.nan
    b = T(bh, cuda)
    L = _lib.lib()
    for lower in (1, 0):
        info = api._ws(L.bilu_sptrsv_analysis_bytes(A.nb), cuda)
        ws = api._ws(max(L.bilu_sptrsv_analysis_ws_bytes(A.nb, A.nnzb),
                         L.bilu_sptrsv_solve_ws_bytes(A.nb)), cuda)
        api.call("bilu_sptrsv_analysis", A.nb, A.nnzb, A.bs, api._p(row), api._p(col), lower,
                 api._p(info), api._p(ws), ws.numel(), api._s())
        xs = []
        for fn in ("bilu_sptrsv_solve_level", "bilu_sptrsv_solve_syncfree"):
            x = torch.empty_like(b)
            api.call(fn, A.nb, A.bs, api._p(row), api._p(col), api._p(lu), lower, lower,
                     api._p(info), api._p(b), api._p(x), api._p(ws), ws.numel(), api._s())
            xs.append(N(x))
        nan0, nan1 = np.isnan(xs[0]), np.isnan(xs[1])
        assert nan0.any() and np.array_equal(nan0, nan1)
        assert np.array_equal(xs[0][~nan0], xs[1][~nan1])


# ------------------------------------------------------------------ errors
def test_pattern_errors(cuda):
    import torch
    from isai_kernel_gb300 import api
    from isai_kernel_gb300._lib import BiluError

    row = T(np.array([0, 2, 3], np.int32), cuda)
    col = T(np.array([1, 0, 0], np.int32), cuda)  # row 0 unsorted
    with pytest.raises(BiluError) as e:
        api.build_bcsc_pattern_from_bsr_scalarILU(2, row, col, True)
    assert e.value.status == -2
    # missing diagonal block in row 1
    row = T(np.array([0, 1, 2], np.int32), cuda)
    col = T(np.array([0, 0], np.int32), cuda)
    val = torch.ones((2, 4, 4), dtype=torch.float64, device=cuda)
    with pytest.raises(BiluError) as e:
        api.bsrilu02_inplace(2, 2, 4, row, col, val)
    assert e.value.status == -2
    # map mismatch reports the first missing (row, col) like the reference
    cp = T(np.array([0, 2, 3], np.int32), cuda)
    ci = T(np.array([0, 1, 1], np.int32), cuda)
    rp = T(np.array([0, 1, 2], np.int32), cuda)
    rc = T(np.array([0, 1], np.int32), cuda)
    with pytest.raises(BiluError) as e:
        api.build_map_bcsc2bcsr_host(2, cp, ci, rp, rc)
    assert e.value.status == -2 and e.value.bad == (1, 0)


def test_zero_pivot_reported(cuda, orc):
    from isai_kernel_gb300 import api

    # block row 0 has no lower neighbour, so its diagonal block reaches the
    # pivot step untouched
    A =gen.laplace2d(4, bs=4, seed=0)
    d = [p for p in range(A.rowptr[0], A.rowptr[1]) if A.colind[p] == 0][0]
    A.val[d][2, :] = 0.0  # scalar row 2 of block row 0: zero pivot u_22
    _, zp = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    v = T(A.val, cuda).clone()
    info = api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), v)
    assert info == zp == 0


def test_single_block_and_empty_offdiag(cuda, orc):
    from isai_kernel_gb300 import api

    rng = np.random.default_rng(0)
    val = rng.uniform(-1, 1, (1, 8, 8)) + 8 * np.eye(8)
    row, col = np.array([0, 1], np.int32), np.array([0], np.int32)
    p = api.Preconditioner(1, 8, T(row, cuda), T(col, cuda), T(val, cuda))
    b = rng.uniform(-1, 1, 8)
    x, res = p.solve(T(b, cuda))
    assert res.converged and res.iters <= 2
    assert np.allclose(val[0] @ N(x), b, atol=1e-10)
    p.close()


# ------------------------------------------------------------------ engine + GMRES
@pytest.mark.parametrize("name", ["c1_s16", "c2_s6", "c3_nb200", "bs5_s7", "long_rows", "dense"])
@pytest.mark.parametrize("schedule", [-1, 0, 1])
def test_engine_factor_match_lists(cuda, orc, name, schedule):
    """A handle's setup builds BILU(0)'s match lists from the pattern before
    a level-order factorisation (a thread per dependency, a warp for the
    ones with more than 32 candidates); its factor is the same bit for bit
    as the entry point that searches for the matches inside the
    factorisation (bsrilu02_inplace, same schedule: recommended, level
    order, sync-free), on short-row, long-row and dense patterns, and within
    1e-12 of the oracle."""
    from isai_kernel_gb300 import api

    if name == "long_rows":
        A = gen.powerlaw(400, bs=8, seed=5, kmax=150)
    elif name == "dense":
        nb, bs = 40, 4
        rng = np.random.default_rng(17)
        val = rng.uniform(-1.0, 1.0, (nb * nb, bs, bs))
        for i in range(nb):
            val[i * nb + i] += np.eye(bs) * (4.0 * nb)
        A = gen.BSRMatrix(nb, bs, (np.arange(nb + 1) * nb).astype(np.int32),
                          np.tile(np.arange(nb, dtype=np.int32), nb), val)
    else:
        A = mats()[name]
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    lu0 = T(A.val, cuda).clone()
    assert api.bsrilu02_inplace(A.nb, A.nnzb, A.bs, row, col, lu0, schedule=schedule) == -1
    p = api.Preconditioner(A.nb, A.bs, row, col, T(A.val, cuda), fp32=False, ilu=True,
                           schedule=schedule)
    lu = N(p.get(0)).reshape(LU.shape)
    p.close()
    assert relerr(lu, LU) < 1e-12
    assert np.array_equal(lu.ravel(), N(lu0).ravel())


@pytest.mark.parametrize("name", ["c1_s16", "c2_s6", "c3_nb200"])
def test_engine_setup_matches_oracle(cuda, orc, name):
    from isai_kernel_gb300 import api

    A = mats()[name]
    S = orc.isai_setup(A)
    p = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda))
    lu, L, U = p.factors()
    assert relerr(N(lu), S["LU"]) < 1e-12
    assert np.array_equal(N(L[0]), S["TrowL"]) and np.array_equal(N(L[1]), S["TcolL"])
    assert np.array_equal(N(U[0]), S["TrowU"]) and np.array_equal(N(U[1]), S["TcolU"])
    assert relerr(N(L[2]), S["McsrL"]) < 1e-12 and relerr(N(U[2]), S["McsrU"]) < 1e-12
    assert np.array_equal(N(p.get(7)), N(L[2]).astype(np.float32).ravel())
    p.close()


@pytest.mark.parametrize("name", ["c1_s16", "c2_s6"])
def test_gmres_iterations_match_oracle(cuda, orc, name):
    from isai_kernel_gb300 import api

    A = mats()[name]
    S = orc.isai_setup(A)
    b = gen.rhs(A.n, 0)
    Ab = (A.rowptr, A.colind, A.val)
    Lo = (S["TrowL"], S["TcolL"], S["McsrL"])
    Uo = (S["TrowU"], S["TcolU"], S["McsrU"])
    xo, ito, rro, ho, st = orc.gmres(Ab, Lo, Uo, b, precond=1, maxit=3000)
    assert st == 0
    p = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda))
    x, res = p.solve(T(b, cuda), prec=0, maxit=3000, history=True)
    assert res.converged and res.iters == ito
    assert relerr(N(x), xo) < 1e-8
    np.testing.assert_allclose(res.history, ho, rtol=1e-6)
    # mixed precision: FP32-stored ISAI inside FP64 FGMRES
    xm, resm = p.solve(T(b, cuda), prec=1, maxit=3000)
    _, itm, _, _, stm = orc.gmres(Ab, Lo, Uo, b, precond=2, maxit=3000)
    assert resm.converged and resm.relres <= 1e-10 and abs(resm.iters - itm) <= 2
    # reproducible
    x2, res2 = p.solve(T(b, cuda), prec=0, maxit=3000)
    assert res2.iters == res.iters and np.array_equal(N(x2), N(x))
    e, r = api.compute_rel_errors(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda),
                                  T(A.val, cuda), T(b, cuda), None, x)
    assert r <= 1.01e-10
    p.close()


@pytest.mark.parametrize("name", ["c1_s16", "c2_s6", "c3_nb200", "bs5_s7"])
def test_gmres_exact_ilu_and_switch(cuda, orc, name):
    """BILU_ILU: z = U^-1 L^-1 v by the level-scheduled triangular solves;
    the iteration count equals the oracle's exact-ILU GMRES, x within 1e-8.
    bilu_ctx_select then returns one of the built choices with positive
    scores, and solve(prec="auto") converges."""
    from isai_kernel_gb300 import api

    A = mats()[name]
    LU, _ = orc.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
    b = gen.rhs(A.n, 0)
    Ab = (A.rowptr, A.colind, A.val)
    xo, ito, rro, ho, st = orc.gmres(Ab, (A.rowptr, A.colind, LU), None, b, precond=3,
                                     maxit=3000)
    assert st == 0
    p = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda),
                           ilu=True, fp32_inner=True, ilu_fp32=True)
    x, res = p.solve(T(b, cuda), prec=api.BILU_ILU, maxit=3000, history=True)
    assert res.converged and res.iters == ito
    assert relerr(N(x), xo) < 1e-8
    np.testing.assert_allclose(res.history, ho, rtol=1e-6)
    # FP32 ISAI + FP32-stored A in the Arnoldi products, FP64 restarts: the
    # oracle's mode 4 within 3 iterations, true residual 1e-10
    S = orc.isai_setup(A)
    Lo = (S["TrowL"], S["TcolL"], S["McsrL"])
    Uo = (S["TrowU"], S["TcolU"], S["McsrU"])
    _, it4, _, _, st4 = orc.gmres(Ab, Lo, Uo, b, precond=4, maxit=3000)
    assert st4 == 0
    x4, res4 = p.solve(T(b, cuda), prec=api.BILU_FP32_INNER, maxit=3000)
    assert res4.converged and res4.relres <= 1e-10 and abs(res4.iters - it4) <= 3
    # exact BILU(0) applied in FP32 on the FP32 factor: FP64 true residual
    # 1e-10 within 3 iterations of the FP64 exact ILU
    x5, res5 = p.solve(T(b, cuda), prec=api.BILU_ILU_FP32, maxit=3000)
    assert res5.converged and res5.relres <= 1e-10 and abs(res5.iters - ito) <= 3
    assert relerr(N(x5), xo) < 1e-8
    choice, rate = p.select(T(b, cuda), cycles=1)
    assert choice in (0, 1, 2, 3, 4) and len(rate) == 5 and all(r > 0 for r in rate)
    xa, resa = p.solve(T(b, cuda), prec="auto", maxit=3000)
    assert resa.converged
    p.close()
    # a handle built without the ILU analyses refuses BILU_ILU
    q = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda))
    with pytest.raises(api.BiluError):
        q.solve(T(b, cuda), prec=api.BILU_ILU)
    q.close()


@pytest.mark.parametrize("name,level", [("c2_s6", 2), ("c2_s6", 3), ("c1_s16", 2),
                                        ("c3_nb200", 2), ("bs5_s7", 2)])
def test_isai_level_k(cuda, orc, name, level):
    """ISAI(k): pattern(A^k) by the symbolic product kernel equals the
    oracle's bit for bit; the engine's M_L / M_U (patterns bit-exact, values
    within 1e-12) equal the oracle's ISAI(k); FP64 GMRES takes the oracle's
    iteration count."""
    from isai_kernel_gb300 import api

    A = mats()[name]
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    pr, pc = row, col
    for _ in range(level - 1):
        pr, pc = api.pattern_product(A.nb, pr, pc, row, col)
    opr, opc = orc.pattern_power(A.nb, A.rowptr, A.colind, level)
    assert np.array_equal(N(pr), opr) and np.array_equal(N(pc), opc)
    S = orc.isai_setup(A, level=level)
    p = api.Preconditioner(A.nb, A.bs, row, col, T(A.val, cuda), isai_level=level)
    lu, Lf, Uf = p.factors()
    assert np.array_equal(N(Lf[0]), S["TrowL"]) and np.array_equal(N(Lf[1]), S["TcolL"])
    assert np.array_equal(N(Uf[0]), S["TrowU"]) and np.array_equal(N(Uf[1]), S["TcolU"])
    assert relerr(N(Lf[2]), S["McsrL"]) < 1e-12 and relerr(N(Uf[2]), S["McsrU"]) < 1e-12
    b = gen.rhs(A.n, 0)
    _, ito, _, _, st = orc.gmres((A.rowptr, A.colind, A.val), (S["TrowL"], S["TcolL"], S["McsrL"]),
                                 (S["TrowU"], S["TcolU"], S["McsrU"]), b, precond=1, maxit=3000)
    assert st == 0
    x, res = p.solve(T(b, cuda), prec=0, maxit=3000)
    assert res.converged and res.iters == ito
    p.close()


def test_pattern_product_too_dense_is_reported(cuda):
    """A row of pattern(A^3) of the power-law system gathers more than 1024
    candidate columns: the kernel reports BILU_ERR_UNSUPPORTED (no
    truncation)."""
    from isai_kernel_gb300 import api

    A = mats()["c3_nb200"]
    row, col = T(A.rowptr, cuda), T(A.colind, cuda)
    p2, c2 = api.pattern_product(A.nb, row, col, row, col)
    with pytest.raises(api.BiluError) as e:
        api.pattern_product(A.nb, p2, c2, row, col)
    assert e.value.status == -8


@pytest.mark.parametrize("name", ["l20", "c3_nb200", "bs5_s7"])
def test_solve_host_end_to_end(cuda, orc, name):
    """bilu_solve_host from pageable and from pinned host buffers (pinned: the
    values copy on a second stream while the setup's structure phase runs,
    and the value phase waits for it), block sizes 4, 8 and 5.  Every mode
    reaches 1e-10; the modes the device path also builds give its bits,
    and the FP64 mode the oracle's iteration count."""
    import torch

    from isai_kernel_gb300 import api

    A = gen.laplace2d(20, bs=4, seed=1) if name == "l20" else mats()[name]
    b = gen.rhs(A.n, 5)
    S = orc.isai_setup(A)
    _, ito, _, _, sto = orc.gmres((A.rowptr, A.colind, A.val), (S["TrowL"], S["TcolL"], S["McsrL"]),
                                  (S["TrowU"], S["TcolU"], S["McsrU"]), b, precond=1, maxit=3000)
    assert sto == 0
    keep = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            for a in (A.rowptr, A.colind, A.val.reshape(-1), b)]
    pinned = [t.numpy() for t in keep]
    stencil = name != "c3_nb200"  # the FP32 exact-ILU apply takes rows of <= 32 dependencies
    P = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda),
                           fp32=True, ilu=True, ilu_fp32=stencil)
    modes = (api.BILU_FP64, api.BILU_FP32, api.BILU_ILU, api.BILU_NESTED)
    for prec in modes + ((api.BILU_ILU_FP32,) if stencil else ()):
        xs = []
        for bufs in ((A.rowptr, A.colind, A.val, b), pinned):
            x, res, times = api.solve_host(A.nb, A.bs, *bufs, prec=prec)
            assert res.converged, prec
            r = b - A.to_dense() @ x
            assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.01e-10
            xs.append(x)
        assert np.array_equal(xs[0], xs[1]), prec
        if prec != api.BILU_NESTED:
            xd, resd = P.solve(T(b, cuda), prec=prec, maxit=10000)
            assert resd.iters == res.iters and np.array_equal(N(xd), xs[0]), prec
        if prec == api.BILU_FP64:
            assert res.iters == ito
    P.close()


def test_solve_host_errors(cuda, orc):
    """bilu_solve_host's failure paths free what the call allocated: a
    missing diagonal block and an unsorted row fail in the setup's structure
    phase (BILU_ERR_PATTERN, before the uploaded values are handed to the
    handle), a solve that stops at maxit returns BILU_ERR_NOT_CONVERGED with
    its last iterate (after the hand-over); calls before and after give the
    same x bit for bit."""
    from isai_kernel_gb300 import api

    A = gen.laplace2d(8, bs=4, seed=0)
    b = gen.rhs(A.n, 2)
    x0, res0, _ = api.solve_host(A.nb, A.bs, A.rowptr, A.colind, A.val, b, prec=api.BILU_NESTED)
    assert res0.converged and res0.relres <= 1e-10
    # row 3 without its diagonal block
    p = int(A.rowptr[3] + np.nonzero(A.colind[A.rowptr[3]:A.rowptr[4]] == 3)[0][0])
    row = A.rowptr.copy()
    row[4:] -= 1
    col = np.delete(A.colind, p)
    val = np.delete(A.val, p, axis=0)
    with pytest.raises(api.BiluError) as e:
        api.solve_host(A.nb, A.bs, row, col, val, b, prec=api.BILU_NESTED)
    assert e.value.status == -2
    # row 5 with two columns swapped
    col = A.colind.copy()
    s5 = int(A.rowptr[5])
    col[s5], col[s5 + 1] = col[s5 + 1], col[s5]
    with pytest.raises(api.BiluError) as e:
        api.solve_host(A.nb, A.bs, A.rowptr, col, A.val, b, prec=api.BILU_FP64)
    assert e.value.status == -2
    x2, res2, _ = api.solve_host(A.nb, A.bs, A.rowptr, A.colind, A.val, b, prec=api.BILU_FP64,
                                 maxit=2)
    assert not res2.converged and res2.iters == 2 and np.all(np.isfinite(x2))
    x3, res3, _ = api.solve_host(A.nb, A.bs, A.rowptr, A.colind, A.val, b, prec=api.BILU_NESTED)
    assert res3.iters == res0.iters and np.array_equal(x3, x0)


@pytest.mark.parametrize("name,inner", [("c1_s16", 10), ("c2_s6", 20), ("c3_nb200", 20),
                                        ("bs5_s7", 8), ("c1_s16", 1), ("c2_s6", 32)])
def test_gmres_nested_matches_oracle(cuda, orc, name, inner):
    """BILU_NESTED (GMRES-IR): FP64 flexible outer GMRES(30) whose every
    preconditioned vector is `inner` steps of FP32 ISAI-preconditioned GMRES
    on the FP32-stored A.  The FP32 inner arithmetic differs from the
    oracle's in rounding only (fused multiply-adds, summation order), so the
    outer iteration count is within 1 of the oracle's nested mode; the FP64
    true residual reaches 1e-10 and x is within 1e-8 of the oracle's FP64
    GMRES solution.  Two solves in a row give the same x bit for bit."""
    from isai_kernel_gb300 import api

    A = mats()[name]
    S = orc.isai_setup(A)
    b = gen.rhs(A.n, 0)
    Ab = (A.rowptr, A.colind, A.val)
    Lo = (S["TrowL"], S["TcolL"], S["McsrL"])
    Uo = (S["TrowU"], S["TcolU"], S["McsrU"])
    x64, _, _, _, st64 = orc.gmres(Ab, Lo, Uo, b, precond=1, maxit=3000)
    xo, ito, inno, rro, _, st = orc.gmres_nested(Ab, Lo, Uo, b, inner=inner, maxit=300)
    assert st == 0 and st64 == 0
    p = api.Preconditioner(A.nb, A.bs, T(A.rowptr, cuda), T(A.colind, cuda), T(A.val, cuda),
                           nested=True, inner=inner)
    x, res = p.solve(T(b, cuda), prec=api.BILU_NESTED, maxit=300)
    assert res.converged and res.relres <= 1e-10
    assert abs(res.iters - ito) <= 1, (res.iters, ito)
    assert res.inner_steps == res.iters * inner
    assert relerr(N(x), x64) < 1e-8 and relerr(N(x), xo) < 1e-8
    x2, res2 = p.solve(T(b, cuda), prec=api.BILU_NESTED, maxit=300)
    assert res2.iters == res.iters and np.array_equal(N(x2), N(x))
    r = b - A.to_dense() @ N(x) if A.n <= 4096 else None
    if r is not None:
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.01e-10
    p.close()


@pytest.mark.parametrize("fp32", [0, 1])
def test_mgs_step_kernel(cuda, fp32):
    """The one-launch Gram-Schmidt step (bilu_debug_mgs_step) against the
    same modified Gram-Schmidt in numpy (FP64) on an orthonormal basis: h
    within 1e-12 relative for FP64 vectors (2e-5 for FP32), v_{j+1} of unit
    norm and orthogonal to the basis, n not a multiple of the vector width
    (the scalar tail), two launches in a row identical bit for bit."""
    import torch

    from isai_kernel_gb300 import _lib, api

    L = _lib.lib()
    n, j = 100003, 6
    ldv = (n + 31) // 32 * 32
    rng = np.random.default_rng(3)
    Vh = np.linalg.qr(rng.standard_normal((n, j + 1)))[0].T  # orthonormal rows
    wh = rng.standard_normal(n)
    dt = torch.float32 if fp32 else torch.float64
    Vp = np.zeros((j + 1, ldv))
    Vp[:, :n] = Vh
    V = torch.from_numpy(Vp.ravel()).to(cuda).to(dt)
    ws = torch.empty(L.bilu_debug_mgs_step_ws_bytes(), dtype=torch.uint8, device=cuda)
    outs = []
    for _ in range(2):
        w = torch.zeros(ldv, dtype=dt, device=cuda)
        w[:n] = torch.from_numpy(wh).to(dt)
        h = torch.empty(j + 2, dtype=torch.float64, device=cuda)
        vn = torch.zeros_like(w)
        st = L.bilu_debug_mgs_step(n, fp32, api._p(V), ldv, j, api._p(w), api._p(h), api._p(vn),
                                   api._p(ws), ws.numel(), api._s())
        assert st == 0
        outs.append((N(h), N(vn)))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    hg, vg = outs[0]
    Vr = N(V).astype(np.float64).reshape(j + 1, ldv)[:, :n]
    wr = N(torch.from_numpy(wh).to(dt)).astype(np.float64)
    href = np.zeros(j + 2)
    for i in range(j + 1):
        href[i] = Vr[i] @ wr
        wr = wr - href[i] * Vr[i]
    href[j + 1] = wr @ wr
    tol = 2e-5 if fp32 else 1e-12
    np.testing.assert_allclose(hg, href, rtol=tol, atol=tol * np.abs(href).max())
    v = vg[:n].astype(np.float64)
    assert abs(np.linalg.norm(v) - 1.0) < (1e-5 if fp32 else 1e-12)
    assert np.abs(Vr @ v).max() < (1e-4 if fp32 else 1e-10)
