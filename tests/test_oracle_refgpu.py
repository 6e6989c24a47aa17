"""Pins the oracle's numeric ISAI steps against the reference's own GPU
kernels (compiled from its sources for sm_103a and run on GB300 by
tests/golden/make_golden_gpu.py): build_DinvL/U_from_BSR5_kernel_fix, the
pair lists of count/fill_pairs_lower_kernel_v2, every ISAI-L variant
(scalar cachedY, bs4 tensor cachedY, bs4 tensor globalY), ISAI-U,
reorder_bcsc_val_to_bcsr_bs5 and the bcsr_spmv apply, all on the same
factor.  Integer outputs bit-exact, values within 1e-12 relative."""
import numpy as np
import pytest

from conftest import golden

CASES = ["refgpu_convdiff3d_s6", "refgpu_laplace2d_s12", "refgpu_powerlaw_nb150"]


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_gpu_kernels(orc, name):
    d = golden(name)
    nb, bs = int(d["nb"]), int(d["bs"])
    row, col, LU = d["row"], d["col"], d["LU"]
    DL = orc.dinv(nb, bs, row, col, LU, True)
    DU = orc.dinv(nb, bs, row, col, LU, False)
    assert rel(DL, d["DinvL"]) < 1e-12 and rel(DU, d["DinvU"]) < 1e-12
    mp, mi = orc.isai_pattern(nb, row, col, True)
    pp, pl, ps = orc.pairs_lower(nb, row, col, mp, mi)
    assert np.array_equal(pp, d["PairPtr"])
    assert np.array_equal(pl, d["PairPLocal"]) and np.array_equal(ps, d["PairSrc"])
    ML = orc.isai_lower(nb, bs, LU, mp, mi, pp, pl, ps, DL)
    variants = [k for k in d if k.startswith("MvalL_")]
    assert variants
    for k in variants:
        assert rel(ML, d[k]) < 1e-12, k
    mpu, miu = orc.isai_pattern(nb, row, col, False)
    MU = orc.isai_upper(nb, bs, row, col, LU, mpu, miu, DU)
    assert rel(MU, d["MvalU"]) < 1e-12
    trL, tcL = orc.tri_pattern(nb, row, col, True)
    trU, tcU = orc.tri_pattern(nb, row, col, False)
    mapL = orc.map_bcsc2bcsr(nb, mp, mi, trL, tcL)
    mapU = orc.map_bcsc2bcsr(nb, mpu, miu, trU, tcU)
    # the reference reordered its own last ISAI-L result and its ISAI-U
    last = d[variants[-1]]
    assert np.array_equal(orc.reorder_bcsc_to_bcsr(bs, mapL, last), d["McsrL"])
    assert np.array_equal(orc.reorder_bcsc_to_bcsr(bs, mapU, d["MvalU"]), d["McsrU"])
    y = orc.bcsr_spmv(nb, bs, trL, tcL, d["McsrL"], d["b"])
    x = orc.bcsr_spmv(nb, bs, trU, tcU, d["McsrU"], y)
    assert rel(x, d["apply_x"]) < 1e-12
