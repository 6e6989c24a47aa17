"""The C++ drop-in layer (include/bilu_isai_compat.hpp): a compiled C++
program (tests/compat_pipeline.cpp) replays the reference's main.cu pipeline
(main.cu:449-866) through the reference's own host entry points -- the
Matrix Market reader, csr_to_bsr5, build_bcsc_pattern_from_bsr_scalarILU,
build_triangular_bcsr_pattern_from_A, build_map_bcsc2bcsr_host,
bsrilu02_inplace, the Dinv / pair / ISAI / reorder steps, the two-SpMV apply,
compute_rel_errors_csr, bsr_SpMV_tensorcore, bsr2csr_cusparse,
csr_cape_SpTRSV and bcsc_to_bcsr -- on libbilu_isai.so, and its outputs are
checked against the CPU oracle: patterns and copies bit-exact, factors,
ISAI values, applies and solves within 1e-12 relative, the residual-check
lines within their printed precision."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from isai_kernel_gb300 import gen

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) if b.size else 0.0


def build_driver(tmp, bs):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.fail("no C++ compiler for the compat driver")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.join(ROOT, "isai_kernel_gb300")
    exe = os.path.join(tmp, f"compat_pipeline_bs{bs}")
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", f"-DCOMPAT_BS={bs}",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "compat_pipeline.cpp"),
           "-L", libdir, "-lbilu_isai", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def write_mtx(path, A):
    row, col, val = A.to_csr()
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{A.n} {A.n} {len(val)}\n")
        for i in range(A.n):
            for p in range(row[i], row[i + 1]):
                f.write(f"{i + 1} {col[p] + 1} {float(val[p])!r}\n")
    return row, col, val


@pytest.mark.parametrize("bs,make", [(4, lambda: gen.laplace2d(16, bs=4, seed=0)),
                                     (4, lambda: gen.convdiff3d(7, bs=4, seed=1)),
                                     (8, lambda: gen.powerlaw(120, bs=8, seed=0, kmax=20))])
def test_compat_pipeline_matches_oracle(cuda, orc, tmp_path, bs, make):
    A = make()
    tmp = str(tmp_path)
    exe = build_driver(tmp, bs)
    mtx = os.path.join(tmp, "A.mtx")
    crow, ccol, cval = write_mtx(mtx, A)
    out = os.path.join(tmp, "out")
    os.makedirs(out)
    r = subprocess.run([exe, mtx, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "compat pipeline ok" in r.stdout
    rd = lambda name, dt: np.fromfile(os.path.join(out, name), dtype=dt)
    S = orc.isai_setup(A)
    LU = rd("lu.f64", np.float64).reshape(-1, bs, bs)
    assert relerr(LU, S["LU"]) < 1e-12
    assert np.array_equal(rd("mbcscL.i32", np.int32), S["MptrL"])
    assert np.array_equal(rd("mindL.i32", np.int32), S["MindL"])
    for t in ("L", "U"):
        assert np.array_equal(rd(f"Mrow{t}.i32", np.int32), S[f"Trow{t}"])
        assert np.array_equal(rd(f"Mcol{t}.i32", np.int32), S[f"Tcol{t}"])
        assert relerr(rd(f"Mval{t}.f64", np.float64), S[f"Mcsr{t}"].ravel()) < 1e-12
    # b = A * 0.7 summed over each CSR row in column order, then the apply
    xt = np.full(A.n, 0.7)
    b = np.array([sum(cval[p] * xt[ccol[p]] for p in range(crow[i], crow[i + 1]))
                  for i in range(A.n)])
    assert np.array_equal(rd("b.f64", np.float64), b)
    xo = orc.bcsr_spmv(A.nb, bs, S["TrowU"], S["TcolU"], S["McsrU"],
                       orc.bcsr_spmv(A.nb, bs, S["TrowL"], S["TcolL"], S["McsrL"], b))
    x = rd("x.f64", np.float64)
    assert relerr(x, xo) < 1e-12
    eo, ro = orc.rel_errors(A.n, crow, ccol, cval, b, xt, xo)
    got = dict(re.findall(r"\] (rel_error_x|rel_residual) = ([0-9.eE+-]+)", r.stdout))
    assert abs(float(got["rel_error_x"]) - eo) <= 1e-5 * eo
    assert abs(float(got["rel_residual"]) - ro) <= 1e-5 * ro
    # bsr_SpMV_tensorcore: A x_true
    ya = orc.bcsr_spmv(A.nb, bs, A.rowptr, A.colind, A.val, xt)
    assert relerr(rd("spmv.f64", np.float64), ya) < 1e-13
    # bsr2csr_cusparse of the factor, then csr_cape_SpTRSV on it
    r_, c_, v_ = orc.bsr_to_csr(A.nb, bs, A.rowptr, A.colind, S["LU"])
    assert np.array_equal(rd("csr_row.i32", np.int32), r_)
    assert np.array_equal(rd("csr_col.i32", np.int32), c_)
    assert relerr(rd("csr_val.f64", np.float64), v_) < 1e-12
    xs = orc.sptrsv_upper(A.nb, bs, A.rowptr, A.colind, S["LU"],
                          orc.sptrsv_lower(A.nb, bs, A.rowptr, A.colind, S["LU"], b))
    assert relerr(rd("cape.f64", np.float64), xs) < 1e-12
    # bcsc_to_bcsr of M_L's BCSC values is the reorder's result
    assert np.array_equal(rd("bcsr_from_bcsc.f64", np.float64), rd("MvalL.f64", np.float64))
