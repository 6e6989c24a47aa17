"""Pins the CPU oracle against golden vectors produced by the reference's own
host code (tests/golden/make_golden.py): every integer array bit-exact,
values bit-exact where the reference copies or sums in a fixed order."""
import numpy as np
import pytest

from conftest import golden

MATS = ["laplace2d_s12", "convdiff3d_s5", "powerlaw_nb120", "laplace2d_s9_bs5"]


@pytest.mark.parametrize("bs", [4, 5, 8])
def test_csr_to_bsr_messy_input(orc, bs):
    g = golden(f"c2b_bs{bs}")
    row, col, val = orc.csr_to_bsr(int(g["n"]), bs, g["csr_row"], g["csr_col"], g["csr_val"])
    assert np.array_equal(row, g["bsr_row"])
    assert np.array_equal(col, g["bsr_col"])
    assert np.array_equal(val, g["bsr_val"])  # duplicates summed in the same order


@pytest.mark.parametrize("name", MATS)
def test_patterns_and_map(orc, name):
    g = golden(name)
    nb = int(g["nb"])
    for lower, tag in ((True, "L"), (False, "U")):
        mp, mi = orc.isai_pattern(nb, g["row"], g["col"], lower)
        assert np.array_equal(mp, g[f"Mptr{tag}"]) and np.array_equal(mi, g[f"Mind{tag}"])
        tr, tc = orc.tri_pattern(nb, g["row"], g["col"], lower)
        assert np.array_equal(tr, g[f"Trow{tag}"]) and np.array_equal(tc, g[f"Tcol{tag}"])
        m = orc.map_bcsc2bcsr(nb, mp, mi, tr, tc)
        assert np.array_equal(m, g[f"map{tag}"])


@pytest.mark.parametrize("name", MATS)
def test_spmv_and_roundtrip(orc, name):
    g = golden(name)
    nb, bs = int(g["nb"]), int(g["bs"])
    y = orc.bcsr_spmv(nb, bs, g["row"], g["col"], g["val"], g["x"])
    assert np.array_equal(y, g["spmv_y"])  # same summation order as cpu_bcsr_spmv
    # CSR -> BSR of the scalar expansion returns the original blocks
    crow, ccol, cval = orc.bsr_to_csr(nb, bs, g["row"], g["col"], g["val"])
    row, col, val = orc.csr_to_bsr(nb * bs, bs, crow, ccol, cval)
    assert np.array_equal(row, g["c2b_row"]) and np.array_equal(col, g["c2b_col"])
    assert np.array_equal(val, g["c2b_val"])


@pytest.mark.parametrize("name", MATS)
def test_bcsc_values_reorder_matches_bcsc_matvec(orc, name):
    """Values in BCSC order, moved to BCSR by the map, give the reference's
    BCSC matvec (spmv_debug.h:44) through the BCSR SpMV."""
    g = golden(name)
    nb, bs = int(g["nb"]), int(g["bs"])
    vals = orc.reorder_bcsc_to_bcsr(bs, g["mapL"], g["bcsc_val"])
    y = orc.bcsr_spmv(nb, bs, g["TrowL"], g["TcolL"], vals, g["x"])
    np.testing.assert_allclose(y, g["bcsc_y"], rtol=1e-13, atol=1e-13)
    # and the deterministic BCSC->BCSR conversion gives the same matrix
    rp, ci, v = orc.bcsc_to_bcsr(nb, nb, bs, g["MptrL"], g["MindL"], g["bcsc_val"])
    assert np.array_equal(rp, g["TrowL"]) and np.array_equal(ci, g["TcolL"])
    assert np.array_equal(v, vals)


def test_mtx_reader_matches_generator(orc):
    g = golden("mtx")
    from isai_kernel_gb300 import gen

    A = gen.laplace2d(4, bs=4, seed=3)
    rp, ci, v = A.to_csr()
    assert int(g["nrows"]) == A.n and int(g["ncols"]) == A.n
    assert np.array_equal(g["row"], rp) and np.array_equal(g["col"], ci)
    assert np.array_equal(g["val"], v)
