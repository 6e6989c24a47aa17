"""This library's GPU kernels against the reference's own GPU kernels
(golden vectors recorded on GB300 by tests/golden/make_golden_gpu.py):
Dinv, pair lists, ISAI-L/U values, the BCSC->BCSR reorder and the
two-SpMV apply on the same factor.  Pair lists bit-exact, values within
1e-12 relative."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

CASES = ["refgpu_convdiff3d_s6", "refgpu_laplace2d_s12", "refgpu_powerlaw_nb150"]


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_gpu_kernels(cuda, orc, name):
    import torch

    from isai_kernel_gb300 import api

    d = golden(name)
    nb, bs = int(d["nb"]), int(d["bs"])
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    N = lambda t: t.cpu().numpy()
    row, col, LU = T(d["row"]), T(d["col"]), T(d["LU"])
    DL = api.build_Dinv(nb, bs, row, col, LU, True)
    DU = api.build_Dinv(nb, bs, row, col, LU, False)
    assert rel(N(DL), d["DinvL"]) < 1e-12 and rel(N(DU), d["DinvU"]) < 1e-12
    mp, mi = api.build_bcsc_pattern_from_bsr_scalarILU(nb, row, col, True)
    pp, pl, ps, _ = api.build_pairs(nb, row, col, mp, mi, True)
    assert np.array_equal(N(pp), d["PairPtr"])
    assert np.array_equal(N(pl), d["PairPLocal"]) and np.array_equal(N(ps), d["PairSrc"])
    ML = api.isai_compute(nb, bs, LU, mp, mi, pp, pl, ps, DL, True)
    for k in [k for k in d if k.startswith("MvalL_")]:
        assert rel(N(ML), d[k]) < 1e-12, k
    mpu, miu = api.build_bcsc_pattern_from_bsr_scalarILU(nb, row, col, False)
    ppu, plu, psu, _ = api.build_pairs(nb, row, col, mpu, miu, False)
    MU = api.isai_compute(nb, bs, LU, mpu, miu, ppu, plu, psu, DU, False)
    assert rel(N(MU), d["MvalU"]) < 1e-12
    trL, tcL = api.build_triangular_bcsr_pattern_from_A(nb, row, col, True)
    trU, tcU = api.build_triangular_bcsr_pattern_from_A(nb, row, col, False)
    mapL = api.build_map_bcsc2bcsr_host(nb, mp, mi, trL, tcL)
    mapU = api.build_map_bcsc2bcsr_host(nb, mpu, miu, trU, tcU)
    # the reference reordered its own last ISAI-L variant and its ISAI-U
    last = [k for k in d if k.startswith("MvalL_")][-1]
    Lr = api.reorder_bcsc_val_to_bcsr(mapL, T(d[last]))
    Ur = api.reorder_bcsc_val_to_bcsr(mapU, T(d["MvalU"]))
    assert np.array_equal(N(Lr), d["McsrL"]) and np.array_equal(N(Ur), d["McsrU"])
    x = api.isai_apply(nb, bs, (trL, tcL, Lr), (trU, tcU, Ur), T(d["b"]), prec=0)
    assert rel(N(x), d["apply_x"]) < 1e-12
