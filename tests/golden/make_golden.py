"""Generates the golden fixtures in this directory from the reference itself.

Runs the reference's own host code (csr_to_bsr5, the ISAI / triangular
pattern builders, the BCSC->BCSR map, cpu_bcsr_spmv, the BCSC debug matvec and
the Matrix Market reader of gmfff/isai_kernel), compiled from the reference
sources by `make -C oracle ref` into oracle/_ref/libref_bs<N>.so, on seeded
inputs, and stores inputs and outputs as .npz files.  The CPU oracle is pinned
against these files by tests/test_oracle_golden.py.

Usage (needs the reference tree, so it runs on the build host only):
    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from isai_kernel_gb300 import gen  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
P = ctypes.c_void_p


def ref(bs):
    L = ctypes.CDLL(os.path.join(REF, f"libref_bs{bs}.so"))
    assert L.ref_block_size() == bs
    return L


def ptr(a):
    return a.ctypes.data_as(P)


def i32(a):
    return np.ascontiguousarray(a, np.int32)


def f64(a):
    return np.ascontiguousarray(a, np.float64)


def messy_csr(n, bs, seed):
    """Random CSR with unsorted columns and duplicate entries in some rows."""
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for r in range(n):
        k = int(rng.integers(1, 7))
        c = list(rng.integers(0, n, size=k)) + [r]
        if rng.random() < 0.3:
            c.append(c[0])  # duplicate
        rng.shuffle(c)
        rows += [r] * len(c)
        cols += c
    rows, cols = np.array(rows), np.array(cols)
    rp = np.zeros(n + 1, np.int32)
    np.cumsum(np.bincount(rows, minlength=n), out=rp[1:])
    val = rng.uniform(-1, 1, size=len(cols))
    return rp, i32(cols), f64(val)


def run_csr_to_bsr(L, n, rp, ci, v):
    cap = len(ci) + 8
    bs = L.ref_block_size()
    br = np.zeros(n // bs + 1, np.int32)
    bc = np.zeros(cap, np.int32)
    bv = np.zeros(cap * bs * bs)
    nnzb = L.ref_csr_to_bsr(n, ptr(rp), ptr(ci), ptr(v), len(ci), ptr(br), ptr(bc), ptr(bv), cap)
    return br, bc[:nnzb], bv[: nnzb * bs * bs].reshape(nnzb, bs, bs)


def run_patterns(L, nb, Ar, Ac):
    out = {}
    cap = len(Ac) + nb + 8
    for lower, tag in ((1, "L"), (0, "U")):
        mp = np.zeros(nb + 1, np.int32)
        mi = np.zeros(cap, np.int32)
        k = L.ref_isai_pattern(nb, ptr(Ar), ptr(Ac), lower, ptr(mp), ptr(mi), cap)
        tr = np.zeros(nb + 1, np.int32)
        tc = np.zeros(cap, np.int32)
        kt = L.ref_tri_pattern(nb, ptr(Ar), ptr(Ac), lower, ptr(tr), ptr(tc), cap)
        out[f"Mptr{tag}"], out[f"Mind{tag}"] = mp, mi[:k].copy()
        out[f"Trow{tag}"], out[f"Tcol{tag}"] = tr, tc[:kt].copy()
        if k == kt:
            m = np.zeros(k, np.int32)
            L.ref_map_bcsc2bcsr(nb, ptr(mp), ptr(out[f"Mind{tag}"]), ptr(tr),
                                ptr(out[f"Tcol{tag}"]), ptr(m))
            out[f"map{tag}"] = m
    return out


def main():
    cases = {}
    # 1) csr -> bsr on messy CSR input, every built block size
    for bs in (4, 5, 8):
        L = ref(bs)
        n = bs * 37
        rp, ci, v = messy_csr(n, bs, seed=100 + bs)
        br, bc, bv = run_csr_to_bsr(L, n, rp, ci, v)
        cases[f"c2b_bs{bs}"] = dict(n=n, bs=bs, csr_row=rp, csr_col=ci, csr_val=v, bsr_row=br,
                                    bsr_col=bc, bsr_val=bv)
    # 2) patterns, map, cpu_bcsr_spmv and the BCSC matvec on the workload families
    mats = {
        "laplace2d_s12": gen.laplace2d(12, bs=4, seed=0),
        "convdiff3d_s5": gen.convdiff3d(5, bs=4, seed=0),
        "powerlaw_nb120": gen.powerlaw(120, bs=8, seed=0, kmax=20),
        "laplace2d_s9_bs5": gen.laplace2d(9, bs=5, seed=1),
    }
    for name, A in mats.items():
        L = ref(A.bs)
        Ar, Ac, Av = i32(A.rowptr), i32(A.colind), f64(A.val)
        d = dict(nb=A.nb, bs=A.bs, row=Ar, col=Ac, val=Av)
        d.update(run_patterns(L, A.nb, Ar, Ac))
        x = np.random.default_rng(7).uniform(-1, 1, A.n)
        y = np.zeros(A.n)
        L.ref_cpu_bcsr_spmv(A.nb, ptr(Ar), ptr(Ac), ptr(Av), ptr(x), ptr(y))
        d["x"], d["spmv_y"] = x, y
        # BCSC matvec over the lower ISAI pattern with seeded block values
        mvals = np.random.default_rng(8).uniform(-1, 1, (len(d["MindL"]), A.bs, A.bs))
        yb = np.zeros(A.n)
        L.ref_bcsc_matvec(A.nb, ptr(d["MptrL"]), ptr(d["MindL"]), ptr(f64(mvals)), ptr(x), ptr(yb))
        d["bcsc_val"], d["bcsc_y"] = mvals, yb
        # the reference's CSR->BSR round trip of the same matrix
        crp, cci, cv = A.to_csr()
        br, bc, bv = run_csr_to_bsr(L, A.n, crp, cci, cv)
        d["c2b_row"], d["c2b_col"], d["c2b_val"] = br, bc, bv
        cases[name] = d
    # 3) Matrix Market reader on a file written by the generator
    A = gen.laplace2d(4, bs=4, seed=3)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "a.mtx")
        gen.write_mtx(path, A)
        L = ref(4)
        cap = A.nnzb * 16 + 8
        nr, nc = ctypes.c_int(0), ctypes.c_int(0)
        rp = np.zeros(A.n + 1, np.int32)
        ci = np.zeros(cap, np.int32)
        v = np.zeros(cap)
        k = L.ref_read_mtx(path.encode(), ctypes.byref(nr), ctypes.byref(nc), ptr(rp), ptr(ci),
                           ptr(v), cap)
        text = open(path).read()
    cases["mtx"] = dict(text=np.frombuffer(text.encode(), np.uint8), nrows=nr.value,
                        ncols=nc.value, row=rp, col=ci[:k], val=v[:k])
    for name, d in cases.items():
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        print("wrote", name)


if __name__ == "__main__":
    main()
