"""Golden vectors from the reference's own GPU kernels, and their sm_103a
timings on the 128^3 workload.

Needs oracle/_ref/ref_kernels_bs{4,8}.cubin (`make -C oracle ref refgpu`,
built where the reference tree is) and oracle/libref_gpu_harness.so
(`make -C oracle refharness`), and a GPU.  For each case it runs, with the
launch configurations of main.cu:51-447 and 655-846, the reference's
build_DinvL/U_from_BSR5_kernel_fix, count/fill_pairs_lower_kernel_v2,
the ISAI-L kernels (scalar cachedY, bs4 tensor cachedY and globalY),
isai_upper_bsr5_warpcol_with_Dinv_kernel, reorder_bcsc_val_to_bcsr_bs5 and
bcsr_spmv on a factor computed by the CPU oracle, and writes inputs and
outputs to OUT/refgpu_<case>.npz.

    python tests/golden/make_golden_gpu.py OUT_DIR            # fixtures
    python tests/golden/make_golden_gpu.py OUT_DIR --time 128 # + timings JSON
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from isai_kernel_gb300 import gen  # noqa: E402
from oracle import oracle  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


class RefKernels:
    def __init__(self, bs, slot):
        import torch

        self.torch = torch
        self.H = ctypes.CDLL(os.path.join(ROOT, "oracle", "libref_gpu_harness.so"))
        self.H.refk_load.restype = ctypes.c_int
        self.H.refk_launch.restype = ctypes.c_int
        torch.cuda.init()
        torch.zeros(1, device="cuda")
        self.slot = slot
        rc = self.H.refk_load(slot, os.path.join(REF, f"ref_kernels_bs{bs}.cubin").encode())
        assert rc == 0, f"refk_load failed: {rc}"
        self.names = open(os.path.join(REF, f"ref_kernels_bs{bs}.names")).read().split()

    def mangled(self, name):
        pre = f"_Z{len(name)}{name}"
        hits = [n for n in self.names if n.startswith(pre)]
        assert len(hits) == 1, (name, hits)
        return hits[0]

    def launch(self, name, grid, block, smem, *args):
        keep, ptrs = [], []
        for a in args:
            if isinstance(a, self.torch.Tensor):
                v = ctypes.c_void_p(a.data_ptr())
            else:
                v = ctypes.c_int(int(a))
            keep.append(v)
            ptrs.append(ctypes.cast(ctypes.pointer(v), ctypes.c_void_p))
        arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
        st = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        rc = self.H.refk_launch(self.slot, self.mangled(name).encode(), grid, block, smem, st, arr)
        assert rc == 0, (name, rc)


def run_reference(K, A, LU, bs, timing_reps=0):
    """The reference's ISAI pipeline (main.cu:655-846) on the factor LU."""
    torch = K.torch
    dev = "cuda"
    nb, bs2 = A.nb, bs * bs
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    Ar, Ac, Av = T(A.rowptr), T(A.colind), T(LU)
    out = {}
    mpL, miL = oracle.isai_pattern(nb, A.rowptr, A.colind, True)
    mpU, miU = oracle.isai_pattern(nb, A.rowptr, A.colind, False)
    trL, tcL = oracle.tri_pattern(nb, A.rowptr, A.colind, True)
    trU, tcU = oracle.tri_pattern(nb, A.rowptr, A.colind, False)
    mapL = oracle.map_bcsc2bcsr(nb, mpL, miL, trL, tcL)
    mapU = oracle.map_bcsc2bcsr(nb, mpU, miU, trU, tcU)
    MbL, McL, MbU, McU = T(mpL), T(miL), T(mpU), T(miU)
    mnnz = int(mpL[-1])
    times = {}

    def timed(key, fn):
        fn()
        if timing_reps:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(timing_reps):
                fn()
            e1.record()
            e1.synchronize()
            times[key] = e0.elapsed_time(e1) / timing_reps

    DinvL = torch.empty(nb * bs2, dtype=torch.float64, device=dev)
    timed("DinvL", lambda: K.launch("build_DinvL_from_BSR5_kernel_fix", (nb + 127) // 128, 128, 0,
                                    nb, Ar, Ac, Av, DinvL))
    cnt = torch.zeros(mnnz + 1, dtype=torch.int32, device=dev)
    timed("count_pairs", lambda: K.launch("count_pairs_lower_kernel_v2", nb, 32, 0, nb, Ar, Ac,
                                          MbL, McL, cnt))
    c = cnt.cpu().numpy().astype(np.int64)
    c[-1] = 0
    pp = np.zeros(mnnz + 1, np.int32)
    pp[1:] = np.cumsum(c[:-1])
    total = int(pp[-1])
    PP = T(pp)
    PL = torch.zeros(max(total, 1), dtype=torch.int32, device=dev)
    PS = torch.zeros(max(total, 1), dtype=torch.int32, device=dev)
    timed("fill_pairs", lambda: K.launch("fill_pairs_lower_kernel_v2", nb, 32, 0, nb, Ar, Ac, MbL,
                                         McL, PP, PL, PS))
    nmax = int(np.diff(mpL).max())
    out.update(DinvL=DinvL.cpu().numpy().reshape(nb, bs, bs), PairPtr=pp,
               PairPLocal=PL.cpu().numpy()[:total], PairSrc=PS.cpu().numpy()[:total])
    shm = (2 * bs2 + nmax * bs2) * 8
    variants = [("isai_lower_bsr5_warpcol_with_pairs_kernel_cachedY", True, nb, 32, shm)]
    if bs == 4:
        variants += [("isai_lower_bsr4_warpcol_with_pairs_kernel_cachedY_tensor_notail", True, nb,
                      32, shm),
                     ("isai_lower_bsr4_warpcol_with_pairs_kernel_globalY_tensor_notail", False,
                      (nb + 3) // 4, 128, 4 * 2 * bs2 * 8)]
    ML = None
    for name, has_nmax, g, b, sm in variants:
        M = torch.zeros(mnnz * bs2, dtype=torch.float64, device=dev)
        args = [nb, Ar, Ac, Av, MbL, McL, PP, PL, PS, M, DinvL] + ([nmax] if has_nmax else [])
        timed(name, lambda: K.launch(name, g, b, sm, *args))
        out["MvalL_" + name] = M.cpu().numpy().reshape(mnnz, bs, bs)
        ML = M
    DinvU = torch.empty(nb * bs2, dtype=torch.float64, device=dev)
    timed("DinvU", lambda: K.launch("build_DinvU_from_BSR5_kernel_fix", (nb + 127) // 128, 128, 0,
                                    nb, Ar, Ac, Av, DinvU))
    mnnzU = int(mpU[-1])
    MU = torch.zeros(mnnzU * bs2, dtype=torch.float64, device=dev)
    timed("isai_upper", lambda: K.launch("isai_upper_bsr5_warpcol_with_Dinv_kernel",
                                         (nb + 3) // 4, 128, 4 * 3 * bs2 * 8, nb, Ar, Ac, Av, MbU,
                                         McU, MU, DinvU))
    out.update(DinvU=DinvU.cpu().numpy().reshape(nb, bs, bs),
               MvalU=MU.cpu().numpy().reshape(mnnzU, bs, bs))
    LL = torch.empty_like(ML)
    UU = torch.empty_like(MU)
    timed("reorder", lambda: (K.launch("reorder_bcsc_val_to_bcsr_bs5", mnnz, 32, 0, mnnz, T(mapL),
                                       ML, LL),
                              K.launch("reorder_bcsc_val_to_bcsr_bs5", mnnzU, 32, 0, mnnzU,
                                       T(mapU), MU, UU)))
    b = T(gen.rhs(A.n, 3))
    y = torch.zeros_like(b)
    x = torch.zeros_like(b)
    tL, cL, tU, cU = T(trL), T(tcL), T(trU), T(tcU)
    timed("apply_bcsr_spmv_x2", lambda: (
        K.launch("bcsr_spmv", (nb + 127) // 128, 128, 0, nb, bs, bs, tL, cL, LL, b, y),
        K.launch("bcsr_spmv", (nb + 127) // 128, 128, 0, nb, bs, bs, tU, cU, UU, y, x)))
    torch.cuda.synchronize()
    out.update(b=b.cpu().numpy(), apply_x=x.cpu().numpy(), McsrL=LL.cpu().numpy().reshape(mnnz, bs, bs),
               McsrU=UU.cpu().numpy().reshape(mnnzU, bs, bs))
    return out, times


def main():
    out_dir = sys.argv[1]
    os.makedirs(out_dir, exist_ok=True)
    cases = {
        "convdiff3d_s6": (gen.convdiff3d(6, bs=4, seed=0), 4),
        "laplace2d_s12": (gen.laplace2d(12, bs=4, seed=1), 4),
        "powerlaw_nb150": (gen.powerlaw(150, bs=8, seed=2, kmax=20), 8),
    }
    kernels = {}
    for name, (A, bs) in cases.items():
        if bs not in kernels:
            kernels[bs] = RefKernels(bs, len(kernels))
        LU, zp = oracle.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
        res, _ = run_reference(kernels[bs], A, LU, bs)
        np.savez_compressed(os.path.join(out_dir, f"refgpu_{name}.npz"), nb=A.nb, bs=bs,
                            row=A.rowptr, col=A.colind, LU=LU, **res)
        print("wrote", name)
    if "--time-powerlaw" in sys.argv:
        nbp = int(sys.argv[sys.argv.index("--time-powerlaw") + 1])
        A = gen.powerlaw(nbp, bs=8, seed=0)
        print(json.dumps({"workload": f"powerlaw nb={nbp} bs8 nnzb={A.nnzb}",
                          "factor_and_solve_ms": time_factor_and_solves(A)}))
    if "--time" in sys.argv:
        side = int(sys.argv[sys.argv.index("--time") + 1])
        A = gen.convdiff3d(side, bs=4, seed=0)
        LU, _ = oracle.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
        _, times = run_reference(kernels[4], A, LU, 4, timing_reps=5)
        print(json.dumps({"workload": f"convdiff3d {side}^3 bs4", "reference_kernels_ms": times}))
        print(json.dumps({"workload": f"convdiff3d {side}^3 bs4",
                          "ours_isai_steps_ms": time_our_isai_steps(A, LU, reps=5)}))
        print(json.dumps({"workload": f"convdiff3d {side}^3 bs4",
                          "factor_and_solve_ms": time_factor_and_solves(A)}))


def time_our_isai_steps(A, LU, reps=5):
    """This library's ISAI setup steps on the same factor as the reference
    kernels above, through the C ABI with preallocated outputs (CUDA events,
    mean of `reps` after one warm-up): Dinv, pair lists (count + fill, which
    includes a scan and the host read of the total), ISAI column solves,
    BCSC->BCSR reorder of both factors, and the FP64 / FP32 apply."""
    import torch

    from isai_kernel_gb300 import _lib, api

    L = _lib.lib()
    P = api._p
    dev = "cuda"
    nb, bs, bs2 = A.nb, A.bs, A.bs * A.bs
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    Ar, Ac, Av = T(A.rowptr), T(A.colind), T(LU)
    times = {}

    def timed(key, fn):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        times[key] = e0.elapsed_time(e1) / reps

    side = {}
    for lower, tag in ((1, "L"), (0, "U")):
        mp, mi = oracle.isai_pattern(nb, A.rowptr, A.colind, bool(lower))
        tr, tc = oracle.tri_pattern(nb, A.rowptr, A.colind, bool(lower))
        mp_, mi_ = T(mp), T(mi)
        mnnz = int(mp[-1])
        D = torch.empty(nb * bs2, dtype=torch.float64, device=dev)
        timed(f"Dinv{tag}", lambda: api.call("bilu_build_dinv", nb, bs, P(Ar), P(Ac), P(Av),
                                             lower, P(D), api._s()))
        pp = torch.empty(mnnz + 1, dtype=torch.int32, device=dev)
        ws = api._ws(L.bilu_pairs_ws_bytes(mnnz), dev)
        tot, nmx = ctypes.c_int(0), ctypes.c_int(0)

        def count():
            api.call("bilu_pairs_ptr", nb, P(Ar), P(Ac), P(mp_), P(mi_), lower, P(pp),
                     ctypes.byref(tot), ctypes.byref(nmx), P(ws), ws.numel(), api._s())
        timed(f"count_pairs_{tag}", count)
        pl = torch.empty(max(tot.value, 1), dtype=torch.int32, device=dev)
        ps = torch.empty(max(tot.value, 1), dtype=torch.int32, device=dev)
        timed(f"fill_pairs_{tag}", lambda: api.call("bilu_pairs_fill", nb, P(Ar), P(Ac), P(mp_),
                                                    P(mi_), lower, P(pp), P(pl), P(ps),
                                                    api._s()))
        M = torch.empty(mnnz * bs2, dtype=torch.float64, device=dev)
        timed(f"isai_{tag}", lambda: api.call("bilu_isai_compute", nb, bs, P(Av), P(mp_), P(mi_),
                                              lower, P(pp), P(pl), P(ps), P(D), P(M), api._s()))
        mp_map = T(oracle.map_bcsc2bcsr(nb, mp, mi, tr, tc))
        side[tag] = (mnnz, mp_map, M, torch.empty_like(M), T(tr), T(tc))

    def reorder():
        for tag in ("L", "U"):
            mnnz, mp_map, M, R, _, _ = side[tag]
            api.call("bilu_reorder_bcsc_to_bcsr", mnnz, bs, P(mp_map), P(M), P(R), api._s())
    timed("reorder_L_and_U", reorder)
    b = T(gen.rhs(A.n, 3))
    x = torch.empty_like(b)
    tmp = torch.empty_like(b)
    (_, _, _, RL, trL, tcL), (_, _, _, RU, trU, tcU) = side["L"], side["U"]
    RL32, RU32 = RL.float(), RU.float()
    timed("apply_fp64", lambda: api.call("bilu_isai_apply", nb, bs, 0, P(trL), P(tcL), P(RL),
                                         P(trU), P(tcU), P(RU), P(b), P(tmp), P(x), api._s()))
    timed("apply_fp32", lambda: api.call("bilu_isai_apply", nb, bs, 1, P(trL), P(tcL), P(RL32),
                                         P(trU), P(tcU), P(RU32), P(b), P(tmp), P(x), api._s()))
    return times


def time_factor_and_solves(A, reps=5):
    """cuSPARSE bsrilu02 / bsrsv2 with the reference's settings (bsrilu.h:20,
    BILU_cusparse.h:110-224) beside this library's BILU(0) and sync-free
    solves (level-scheduled and sync-free) on the same matrix (CUDA events,
    GPU time only)."""
    import torch

    from isai_kernel_gb300 import _lib, api

    L = _lib.lib()
    C = ctypes.CDLL(os.path.join(ROOT, "oracle", "libcusparse_ref.so"))
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    dev = "cuda"
    row = torch.from_numpy(A.rowptr).to(dev)
    col = torch.from_numpy(A.colind).to(dev)
    A0 = torch.from_numpy(A.val).to(dev).contiguous()
    out = {}
    ms = (ctypes.c_float * 2)()
    zp = ctypes.c_int(0)
    best = None
    for _ in range(3):
        v = A0.clone()
        C.cusp_bsrilu02(A.nb, A.nnzb, A.bs, P(row), P(col), P(v), ctypes.byref(zp), ms)
        best = (ms[0], ms[1]) if best is None or ms[1] < best[1] else best
    out["cusparse_bsrilu02_analysis_ms"], out["cusparse_bsrilu02_factor_ms"] = best
    lu_ref = v
    ws = api._ws(L.bilu_bsrilu0_ws_bytes(A.nb, A.nnzb), dev)
    ts = []
    for _ in range(3):
        v = A0.clone()
        info = ctypes.c_int(0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        L.bilu_bsrilu0(A.nb, A.nnzb, A.bs, P(row), P(col), P(v), ctypes.byref(info), P(ws),
                       ws.numel(), api._s())
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    out["ours_bilu0_ms_incl_level_analysis"] = min(ts)
    out["factor_max_rel_diff_vs_cusparse"] = float(
        (v - lu_ref).abs().max() / lu_ref.abs().max())
    b = torch.from_numpy(gen.rhs(A.n, 1)).to(dev)
    x = torch.empty_like(b)
    for lower in (1, 0):
        tag = "L" if lower else "U"
        C.cusp_bsrsv2(A.nb, A.nnzb, A.bs, P(row), P(col), P(lu_ref), lower, P(b), P(x), reps, ms)
        out[f"cusparse_bsrsv2_{tag}_analysis_ms"], out[f"cusparse_bsrsv2_{tag}_solve_ms"] = ms[0], ms[1]
        info = torch.empty(L.bilu_sptrsv_analysis_bytes(A.nb), dtype=torch.uint8, device=dev)
        ws = api._ws(max(L.bilu_sptrsv_analysis_ws_bytes(A.nb, A.nnzb),
                         L.bilu_sptrsv_solve_ws_bytes(A.nb)), dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        L.bilu_sptrsv_analysis(A.nb, A.nnzb, A.bs, P(row), P(col), lower, P(info), P(ws),
                               ws.numel(), api._s())
        e1.record()
        e1.synchronize()
        out[f"ours_sptrsv_{tag}_analysis_ms"] = e0.elapsed_time(e1)
        y = torch.empty_like(b)
        L.bilu_sptrsv_solve_level(A.nb, A.bs, P(row), P(col), P(lu_ref), lower, lower, P(info),
                                  P(b), P(y), P(ws), ws.numel(), api._s())
        e0.record()
        for _ in range(reps):
            L.bilu_sptrsv_solve_level(A.nb, A.bs, P(row), P(col), P(lu_ref), lower, lower,
                                      P(info), P(b), P(y), P(ws), ws.numel(), api._s())
        e1.record()
        e1.synchronize()
        out[f"ours_sptrsv_{tag}_level_solve_ms"] = e0.elapsed_time(e1) / reps
        y2 = torch.empty_like(b)
        L.bilu_sptrsv_solve_syncfree(A.nb, A.bs, P(row), P(col), P(lu_ref), lower, lower, P(info),
                                     P(b), P(y2), P(ws), ws.numel(), api._s())
        e0.record()
        for _ in range(reps):
            L.bilu_sptrsv_solve_syncfree(A.nb, A.bs, P(row), P(col), P(lu_ref), lower, lower,
                                         P(info), P(b), P(y2), P(ws), ws.numel(), api._s())
        e1.record()
        e1.synchronize()
        out[f"ours_sptrsv_{tag}_syncfree_solve_ms"] = e0.elapsed_time(e1) / reps
        out[f"sptrsv_{tag}_level_vs_syncfree_identical"] = bool(torch.equal(y, y2))
        out[f"sptrsv_{tag}_max_rel_diff_vs_cusparse"] = float((y - x).abs().max() / x.abs().max())
    return out


if __name__ == "__main__":
    main()
