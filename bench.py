"""Benchmark: block-ILU(0) + ISAI preconditioned GMRES on the 128^3 4-DOF
convection-diffusion system (BSR 4x4, 2,097,152 block rows, 14,581,760
blocks, FP64 matrix), synthetic seeded data.

A step is one solve to 1e-10 relative residual from x0 = 0 with the
mixed-precision path (FP32-stored ISAI inside FP64 flexible GMRES(30) with
FP64 residuals, orthogonalisation and restarts); the preconditioner setup
(BILU(0) + ISAI on the GPU) runs once before the timed region and is
reported separately, as are the plain FP64 ISAI path, the FP32-operator
variant (`fp32_inner`) and GMRES with the exact BILU(0) applied by
level-scheduled triangular solves (`exact_ilu`).  `value` is the mean solve
time (s) with the matrix resident in HBM (1.9 GB of values, larger than L2).
`e2e` is the same metric through the C ABI call with host buffers
(bilu_solve_host: H2D of A and b, setup, solve, D2H of x).  `roofline`
rates the FP32 apply as the solver launches it (two k_bsr_spmv, FP32 basis
vector in) against the measured copy bandwidth; `traffic` is the DRAM bytes
of the same launches from the committed ncu capture.  `cpu_baseline` is the
oracle on the host cores, plus the serial (one core) BILU(0) and triangular
solves.  Secondary lines: --workload sptrsv | powerlaw | batch.

    python bench.py [--steps K] [--warmup W] [--side 128] [--impl reference]
    torchrun --nproc-per-node N bench.py --gpus N   (N independent replicas)
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to 1e-10 rel. residual, mixed vs FP64 BILU-ISAI; precond-apply HBM GB/s"
FALLBACK_HBM_GBS = 6800.0
# FP64 and mixed iteration counts of the 128^3 system measured on GB300 with
# this code (the FP64 count equals the oracle's at every size the oracle can
# finish); used to scale the CPU baseline's per-iteration cost.
C2_ITERS_REF = {"fp64": 328, "mixed": 328}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--side", type=int, default=128)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--restart", type=int, default=30)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--maxit", type=int, default=20000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--workload", default="convdiff",
                    choices=["convdiff", "batch", "powerlaw", "sptrsv"],
                    help="convdiff: the headline line; batch / powerlaw / sptrsv: secondary lines")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-lo", type=int, default=32)
    ap.add_argument("--batch-hi", type=int, default=512)
    ap.add_argument("--batch-rhs", type=int, default=32)
    ap.add_argument("--batch-seed", type=int, default=0)
    ap.add_argument("--batch-mem-gb", type=float, default=160.0)
    ap.add_argument("--pl-nb", type=int, default=500000)
    ap.add_argument("--profile", action="store_true",
                    help="short run for ncu launch lists: setup, one warm-up and one timed "
                         "solve capped at --maxit, the apply loop; no e2e, no CPU baseline")
    a = ap.parse_args()
    if a.profile:
        a.no_cpu_baseline = True
    return a


def probe_lib():
    """bench_probe.so (built by __graft_entry__.build()): pipe-rate and
    synchronisation probes reported beside the numbers."""
    P = ctypes.CDLL(os.path.join(ROOT, "bench_probe.so"))
    for f in (P.probe_rates, P.probe_sync):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(ctypes.c_double)]
    return P


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [ln.split(",") for ln in open(self.f.name).read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, v in zip(names, r[5:9]):
                    if v.strip() == "Active":
                        reasons.add(k)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def apply_bytes(nb, bs, nnzL, nnzU, s_val, s_tmp):
    """Algorithmic bytes of one preconditioner apply y = M_L b, x = M_U y:
    values + column indices of both factors, both row pointers, read b (FP64),
    write and read the intermediate y, write x (FP64)."""
    n = nb * bs
    return (nnzL + nnzU) * (bs * bs * s_val + 4) + 2 * (nb + 1) * 4 + n * (8 + 2 * s_tmp + 8)


def apply_bytes_staged(nb, bs, nnzL, nnzU):
    """Algorithmic bytes of the FP32 apply as the solver runs it (input is
    the FP32 copy of the basis vector written by the normalisation): FP32
    values + column indices, row pointers, read x32, write and read y32,
    write z (FP64)."""
    n = nb * bs
    return (nnzL + nnzU) * (bs * bs * 4 + 4) + 2 * (nb + 1) * 4 + n * (4 + 2 * 4 + 8)


def measured_traffic(side):
    """DRAM bytes per FP32 apply from the committed ncu summary of the same
    workload (profiles/roofline_traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(p):
        return None, None
    d = json.load(open(p))
    if d.get("side") != side:
        return None, None
    return float(d["dram_bytes_per_apply"]), d.get("source")


def spmv_bytes(nb, bs, nnzb):
    n = nb * bs
    return nnzb * (bs * bs * 8 + 4) + (nb + 1) * 4 + 2 * n * 8


def dist_init(args):
    if args.gpus <= 1 and "WORLD_SIZE" not in os.environ:
        return 0, 1
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU baseline
def cpu_baseline(side, iters_full, gmres_iters=3, seed=0):
    """The oracle (plain-C restatement of the reference path, OpenMP over the
    host cores) on the full system: the whole setup (BILU(0), patterns,
    pairs, Dinv, ISAI-L/U, reorder) plus `gmres_iters` FGMRES iterations with
    the FP32-stored ISAI; time to solution = setup + per-iteration cost x
    the solver's iteration count for this system."""
    from isai_kernel_gb300 import gen
    from oracle import oracle

    A = gen.convdiff3d(side, bs=4, seed=seed)
    b = gen.rhs(A.n, seed)
    t0 = time.perf_counter()
    S = oracle.isai_setup(A)
    t_setup = time.perf_counter() - t0
    Ab = (A.rowptr, A.colind, A.val)
    L = (S["TrowL"], S["TcolL"], S["McsrL"])
    U = (S["TrowU"], S["TcolU"], S["McsrU"])
    t0 = time.perf_counter()
    _, it, _, _, _ = oracle.gmres(Ab, L, U, b, precond=2, restart=30, maxit=gmres_iters)
    t_it = (time.perf_counter() - t0) / max(it, 1)
    est = t_setup + t_it * iters_full
    cores = oracle.num_threads()
    # the serial CPU path on one core: BILU(0), the whole ISAI setup (BILU(0)
    # again, patterns, pairs, Dinv, ISAI-L/U, reorder), one FP64 and one
    # FP32-stored apply, the two triangular solves (the reference has no CPU
    # ILU / ISAI / SpTRSV; its GPU kernels are the restated algorithms)
    oracle.set_threads(1)
    try:
        t0 = time.perf_counter()
        LU, _ = oracle.bsrilu0(A.nb, A.bs, A.rowptr, A.colind, A.val)
        t_f1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        y = oracle.sptrsv_lower(A.nb, A.bs, A.rowptr, A.colind, LU, b)
        t_l1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle.sptrsv_upper(A.nb, A.bs, A.rowptr, A.colind, LU, y)
        t_u1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle.isai_setup(A)
        t_s1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        y = oracle.bcsr_spmv(A.nb, A.bs, L[0], L[1], L[2], b)
        oracle.bcsr_spmv(A.nb, A.bs, U[0], U[1], U[2], y)
        t_a64 = time.perf_counter() - t0
        L32, U32, b32 = (a.astype(np.float32) for a in (L[2], U[2], b))
        t0 = time.perf_counter()
        y32 = oracle.bcsr_spmv_f32(A.nb, A.bs, L[0], L[1], L32, b32)
        oracle.bcsr_spmv_f32(A.nb, A.bs, U[0], U[1], U32, y32)
        t_a32 = time.perf_counter() - t0
    finally:
        oracle.set_threads(cores)
    return {"value": est, "unit": "s", "cores": cores, "kind": "port",
            "sample": (f"oracle on the full {side}^3 system: setup {t_setup:.2f} s measured, "
                       f"{it} FGMRES(30) iterations measured at {t_it:.3f} s each, scaled to "
                       f"{iters_full} iterations"),
            "setup_s": t_setup, "per_iter_s": t_it,
            "serial_1_core": {"bilu0_s": t_f1, "isai_setup_s": t_s1, "apply_fp64_s": t_a64,
                              "apply_fp32_s": t_a32, "sptrsv_L_s": t_l1, "sptrsv_U_s": t_u1}}


def run_reference(args):
    rank, world = dist_init(args)
    if rank != 0:
        return
    iters = C2_ITERS_REF["mixed"] or 700
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(args.side, iters, gmres_iters=args.cpu_iters)
        if i >= args.warmup:
            vals.append(r)
    v = statistics.mean(r["value"] for r in vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded 128^3 convection-diffusion, BSR 4x4)",
            "config": {"workload": f"convdiff3d {args.side}^3 bs4, FGMRES(30) tol 1e-10, mixed",
                       "n": args.side ** 3 * 4},
            "cpu_baseline": {"value": v, "unit": "s", "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU arm
def run_ours(args):
    import torch

    from isai_kernel_gb300 import _lib, api, gen

    rank, world = dist_init(args)
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.lib()
    stream = torch.cuda.current_stream()

    A = gen.convdiff3d(args.side, bs=4, seed=0)
    b_np = gen.rhs(A.n, 0)
    nb, bs, nnzb, n = A.nb, A.bs, A.nnzb, A.n
    row = torch.from_numpy(A.rowptr).to(dev)
    col = torch.from_numpy(A.colind).to(dev)
    val = torch.from_numpy(A.val).to(dev)
    b = torch.from_numpy(b_np).to(dev)
    torch.cuda.synchronize()

    P = api.Preconditioner(nb, bs, row, col, val, fp32=True, fp32_inner=True)
    setup_ms = P.setup_ms
    x = torch.empty_like(b)

    def solve(prec):
        return P.solve(b, x, prec=prec, restart=args.restart, tol=args.tol, maxit=args.maxit)

    for _ in range(args.warmup):
        _, res = solve(1)
    barrier(world)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    l0 = L.bilu_kernel_launches()
    times, iters = [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, res = solve(1)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        iters.append(res.iters)
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    launches = L.bilu_kernel_launches() - l0
    relres_mixed = res.relres
    restarts_mixed = res.restarts
    t_mixed = max_over_ranks(statistics.mean(times), world)

    # plain FP64 path (reported beside the headline)
    _, r64 = solve(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _, r64 = solve(0)
    e1.record(stream)
    e1.synchronize()
    t_fp64 = e0.elapsed_time(e1) / 1e3

    # FP32 ISAI plus FP32-stored A in the Arnoldi products (FP64
    # orthogonalisation, true residuals and restarts), reported beside
    _, r32i = solve(3)
    e0.record(stream)
    _, r32i = solve(3)
    e1.record(stream)
    e1.synchronize()
    t_f32i = e0.elapsed_time(e1) / 1e3

    # exact BILU(0) preconditioner (two level-scheduled triangular solves
    # per apply), FP64: reported beside the ISAI paths
    Pi = api.Preconditioner(nb, bs, row, col, val, fp32=False, ilu=True)
    xi = torch.empty_like(b)
    _, ri = Pi.solve(b, xi, prec=api.BILU_ILU, restart=args.restart, tol=args.tol,
                     maxit=args.maxit)
    e0.record(stream)
    _, ri = Pi.solve(b, xi, prec=api.BILU_ILU, restart=args.restart, tol=args.tol,
                     maxit=args.maxit)
    e1.record(stream)
    e1.synchronize()
    t_ilu = e0.elapsed_time(e1) / 1e3
    ilu_setup = Pi.setup_ms["total"]
    Pi.close()
    del Pi
    # the same with the triangular solves in FP32 on an FP32 copy of the factor
    Pf = api.Preconditioner(nb, bs, row, col, val, fp32=False, ilu_fp32=True)
    _, rf = Pf.solve(b, xi, prec=api.BILU_ILU_FP32, restart=args.restart, tol=args.tol,
                     maxit=args.maxit)
    e0.record(stream)
    _, rf = Pf.solve(b, xi, prec=api.BILU_ILU_FP32, restart=args.restart, tol=args.tol,
                     maxit=args.maxit)
    e1.record(stream)
    e1.synchronize()
    t_iluf = e0.elapsed_time(e1) / 1e3
    iluf_setup = Pf.setup_ms["total"]
    Pf.close()
    del Pf, xi

    # preconditioner apply kernels, timed alone with CUDA events on the
    # launching stream (inputs: 1.1-1.9 GB of factors, larger than L2)
    lu, Lf, Uf = P.factors()
    nnzL, nnzU = int(Lf[1].numel()), int(Uf[1].numel())
    L32, U32 = P.get(7).view(-1, bs, bs), P.get(8).view(-1, bs, bs)

    def time_it(fn, reps=20):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    reps = 3 if args.profile else 20
    t_apply64 = time_it(lambda: api.isai_apply(nb, bs, Lf, Uf, b, prec=0), reps)
    t_apply32 = time_it(lambda: api.isai_apply(nb, bs, (Lf[0], Lf[1], L32), (Uf[0], Uf[1], U32),
                                               b, prec=1), reps)
    # the apply as the solver launches it: two k_bsr_spmv, FP32 input and
    # intermediate, FP64 output
    b32 = b.float()
    y32 = torch.empty(n, dtype=torch.float32, device=dev)
    z = torch.empty_like(b)

    def apply_staged():
        L.bilu_bcsr_spmv_f32(nb, bs, api._p(Lf[0]), api._p(Lf[1]), api._p(L32), api._p(b32), 1,
                             api._p(y32), 1, api._s())
        L.bilu_bcsr_spmv_f32(nb, bs, api._p(Uf[0]), api._p(Uf[1]), api._p(U32), api._p(y32), 1,
                             api._p(z), 0, api._s())
    t_apply32s = time_it(apply_staged, reps)
    y = torch.empty_like(b)
    t_spmvA = time_it(lambda: api.bcsr_spmv(nb, bs, row, col, val, b, y), reps)
    B64 = apply_bytes(nb, bs, nnzL, nnzU, 8, 8)
    B32 = apply_bytes(nb, bs, nnzL, nnzU, 4, 4)
    BA = spmv_bytes(nb, bs, nnzb)
    B32s = apply_bytes_staged(nb, bs, nnzL, nnzU)
    peak, peak_kind = peaks()
    gbs32 = B32 / t_apply32 / 1e9
    gbs32s = B32s / t_apply32s / 1e9
    traffic, traffic_src = measured_traffic(args.side)
    rates = (ctypes.c_double * 3)()
    rc = probe_lib().probe_rates(rates)
    assert rc == 0, f"probe_rates returned {rc}"
    dfma_tf = rates[0]
    # FP64 kernels: one DFMA per stored FP64 value, so their compute roofline
    # is 2 * (#values) / DFMA rate
    flops64 = 2.0 * (nnzL + nnzU) * bs * bs
    flopsA = 2.0 * nnzb * bs * bs

    # end to end through the C ABI with pinned host buffers
    hrow = torch.from_numpy(A.rowptr).pin_memory()
    hcol = torch.from_numpy(A.colind).pin_memory()
    hval = torch.from_numpy(A.val).pin_memory()
    hb = torch.from_numpy(b_np).pin_memory()
    hx = torch.empty(n, dtype=torch.float64).pin_memory()
    e2e = []
    for _ in range(0 if args.profile else 2):
        it, rr = ctypes.c_int(0), ctypes.c_double(0)
        tm = (ctypes.c_double * 4)()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = L.bilu_solve_host(nb, nnzb, bs, ctypes.c_void_p(hrow.data_ptr()),
                               ctypes.c_void_p(hcol.data_ptr()), ctypes.c_void_p(hval.data_ptr()),
                               ctypes.c_void_p(hb.data_ptr()), ctypes.c_void_p(hx.data_ptr()), 1,
                               args.restart, args.tol, args.maxit, ctypes.byref(it),
                               ctypes.byref(rr), tm, ctypes.c_void_p(stream.cuda_stream))
        e2e.append(time.perf_counter() - t0)
        assert st == 0, st
    e2e_v = max_over_ranks(min(e2e), world) if e2e else None
    h2d = A.rowptr.nbytes + A.colind.nbytes + A.val.nbytes + b_np.nbytes
    d2h = n * 8

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(args.side, int(statistics.mean(iters)), gmres_iters=args.cpu_iters)
            cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "setup_s",
                                       "per_iter_s", "serial_1_core")}
        except Exception as exc:  # report, never hide
            cpu = {"value": None, "unit": "s", "cores": 0, "kind": "port",
                   "sample": f"failed: {exc}"}
    P.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": t_mixed, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mixed * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded 128^3 7-point convection-diffusion, 4 DOF, BSR 4x4)",
        "config": {"workload": f"convdiff3d {args.side}^3 bs4 (nb={nb}, nnzb={nnzb}), "
                               f"FGMRES({args.restart}) to {args.tol:g}, FP32-stored ISAI",
                   "nb": nb, "nnzb": nnzb, "restart": args.restart, "tol": args.tol,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (1.87 GB of FP64 values)"},
        "iters": {"mixed": int(statistics.mean(iters)), "fp64": r64.iters},
        "restart_cycles": {"mixed": restarts_mixed, "fp64": r64.restarts},
        "relres": {"mixed": relres_mixed, "fp64": r64.relres},
        "fp64_solve_s": t_fp64, "speedup_mixed_vs_fp64": t_fp64 / t_mixed,
        "exact_ilu": {"s": t_ilu, "iters": ri.iters, "relres": ri.relres,
                      "setup_ms": ilu_setup, "speedup_vs_fp64_isai": t_fp64 / t_ilu,
                      "what": "FP64 FGMRES(30) with the exact BILU(0) applied by two "
                              "level-order block triangular solves"},
        "exact_ilu_fp32": {"s": t_iluf, "iters": rf.iters, "relres": rf.relres,
                           "setup_ms": iluf_setup, "speedup_vs_fp64_isai": t_fp64 / t_iluf,
                           "what": "FP64 FGMRES(30) with the exact BILU(0) applied in FP32 "
                                   "(FP32 copy of the factor, FP32 level-order solves)"},
        "fp32_inner": {"s": t_f32i, "iters": r32i.iters, "relres": r32i.relres,
                       "restart_cycles": r32i.restarts, "speedup_vs_fp64": t_fp64 / t_f32i,
                       "what": "FP32 ISAI + FP32-stored A in the Arnoldi products; FP64 "
                               "orthogonalisation, true residual and restarts"},
        "setup_ms": setup_ms,
        "apply": {"fp32_s": t_apply32, "fp64_s": t_apply64, "fp32_GBs": gbs32,
                  "fp32_solver_s": t_apply32s, "fp32_solver_GBs": gbs32s,
                  "fp64_GBs": B64 / t_apply64 / 1e9, "bytes_fp32": B32, "bytes_fp64": B64,
                  "A_spmv_s": t_spmvA, "A_spmv_GBs": BA / t_spmvA / 1e9},
        "roofline": {"bound": "hbm", "achieved": gbs32s, "peak": peak, "unit": "GB/s",
                     "frac": gbs32s / peak, "traffic": traffic,
                     "algorithmic_bytes": B32s, "duration_s": t_apply32s,
                     "kernel": "FP32-stored ISAI apply as run in the solver (k_bsr_spmv x2: "
                               "M_L on the FP32 basis vector, M_U to FP64)",
                     "traffic_source": traffic_src,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "fp64_compute_roofline": {
            "dfma_tflops": dfma_tf, "dmma_tflops": rates[1], "ffma_tflops": rates[2],
            "apply_fp64_frac_of_dfma": flops64 / t_apply64 / 1e12 / dfma_tf,
            "A_spmv_frac_of_dfma": flopsA / t_spmvA / 1e12 / dfma_tf,
            "apply_fp64_bound_s": max(flops64 / (dfma_tf * 1e12), B64 / (peak * 1e9)),
            "A_spmv_bound_s": max(flopsA / (dfma_tf * 1e12), BA / (peak * 1e9))},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk, "wall_s": wall,
    }
    print(json.dumps(line))


def run_batch(args):
    """Secondary line: 256 seeded 2D 5-point 4-DOF systems, grid sides
    U{32..512} (seed s for system s), 32 uniform right-hand sides each, FP32
    ISAI apply inside FP64 FGMRES(30), all systems in one block-diagonal setup
    and per-step single launches; --maxit caps the Arnoldi steps per wave."""
    import torch

    from isai_kernel_gb300 import api, gen

    rng = np.random.default_rng(args.batch_seed)
    sides = rng.integers(args.batch_lo, args.batch_hi + 1, size=args.batch_count)
    mats = [gen.laplace2d(int(s), bs=4, seed=args.batch_seed + i) for i, s in enumerate(sides)]
    k = args.batch_rhs
    B = np.concatenate([gen.rhs(A.n, args.batch_seed + i, k=k) for i, A in enumerate(mats)])
    t0 = time.perf_counter()
    bt = api.Batch(mats)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    Bd = torch.from_numpy(B).cuda()
    X, iters, relres, stats = bt.solve(Bd, restart=args.restart, tol=args.tol, maxit=args.maxit,
                                       mem_budget=int(args.batch_mem_gb * (1 << 30)))
    cfg, tune_ms = bt.tuning()
    conv = float(np.mean(relres <= args.tol))
    line = {"workload": f"batch {args.batch_count} x laplace2d U{{{args.batch_lo}..{args.batch_hi}}}"
                        f" bs4, {k} rhs, FGMRES({args.restart}) FP32 ISAI, maxit {args.maxit}",
            "systems": args.batch_count, "rhs": k, "block_rows": bt.nb,
            "setup_s": t_setup, "solve_s": stats[3] / 1e3, "waves": int(stats[0]),
            "graph_launches": int(stats[1]), "pair_steps": int(stats[2]),
            "pair_steps_per_s": stats[2] / (stats[3] / 1e3),
            "converged_fraction": conv, "median_iters": float(np.median(iters)),
            "autotune": {"rows_per_warp_A": cfg[0], "rows_per_warp_apply": cfg[1],
                         "tile_rows": cfg[2], "candidates_ms_A": tune_ms[:3],
                         "candidates_ms_apply": tune_ms[3:6]}}
    bt.close()
    print(json.dumps(line))


def run_powerlaw(args):
    """Secondary line: random power-law block matrix (500k block rows, 8x8
    blocks), BILU(0)+ISAI setup and FP64 / mixed FGMRES(30) to 1e-10."""
    import torch

    from isai_kernel_gb300 import api, gen

    A = gen.powerlaw(args.pl_nb, bs=8, seed=0)
    b = torch.from_numpy(gen.rhs(A.n, 0)).cuda()
    row, col, val = (torch.from_numpy(a).cuda() for a in (A.rowptr, A.colind, A.val))
    # the first setup grows the library's memory pool (the driver maps
    # ~20 GB, at a cost that differs from box to box); the second one, after
    # the first handle returned its buffers to the pool, times the kernels
    P = api.Preconditioner(A.nb, 8, row, col, val)
    cold = P.setup_ms
    P.close()
    P = api.Preconditioner(A.nb, 8, row, col, val)
    out = {"workload": f"powerlaw nb={A.nb} bs8 nnzb={A.nnzb}", "setup_ms": P.setup_ms,
           "setup_cold_ms": cold}
    for prec, tag in ((0, "fp64"), (1, "mixed")):
        P.solve(b, prec=prec, maxit=args.maxit)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, res = P.solve(b, prec=prec, maxit=args.maxit)
        e1.record()
        e1.synchronize()
        out[tag] = {"s": e0.elapsed_time(e1) / 1e3, "iters": res.iters, "relres": res.relres}
    lu, Lf, Uf = P.factors()
    x = torch.empty_like(b)
    t = []
    for lower in (True, False):
        api.sptrsv(A.nb, 8, row, col, lu.view(-1, 8, 8), b, lower=lower)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        api.sptrsv(A.nb, 8, row, col, lu.view(-1, 8, 8), b, lower=lower)
        e1.record()
        e1.synchronize()
        t.append(e0.elapsed_time(e1))
    out["sptrsv_ms_incl_analysis"] = {"L": t[0], "U": t[1]}
    P.close()
    print(json.dumps(out))


def run_sptrsv(args):
    """Secondary line: block triangular solves with the packed BILU(0) of the
    --side^3 convection-diffusion system.  One level analysis per triangle,
    then the level-scheduled and the sync-free solve on it (CUDA events over
    --steps solves each, after --warmup).  Bytes per solve: the triangle's
    blocks with their column indices, the diagonal blocks, row pointers,
    the order, b and x."""
    import torch

    from isai_kernel_gb300 import _lib, api, gen

    L = _lib.lib()
    A = gen.convdiff3d(args.side, bs=4, seed=0)
    nb, bs, nnzb = A.nb, A.bs, A.nnzb
    dev = torch.device("cuda", 0)
    row, col, val = (torch.from_numpy(a).to(dev) for a in (A.rowptr, A.colind, A.val))
    lu = val.clone()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    zp = api.bsrilu02_inplace(nb, nnzb, bs, row, col, lu)
    e1.record()
    e1.synchronize()
    out = {"workload": f"sptrsv convdiff3d {args.side}^3 bs4 (nb={nb}, nnzb={nnzb})",
           "bilu0_ms_incl_analysis": e0.elapsed_time(e1), "zero_pivot": zp}
    # what the level-order kernels are bound by (SM cycles)
    sp = (ctypes.c_double * 8)()
    rc = probe_lib().probe_sync(sp)
    assert rc == 0, f"probe_sync returned {rc}"
    out["sync_probe_cycles"] = {
        "dfma_interval_per_sm_1_4_16_warps": [round(sp[0], 1), round(sp[1], 1), round(sp[2], 1)],
        "dfma_interval_per_sm_4_warps_4_lanes": round(sp[3], 1),
        "store_to_load_one_way_min_max": [round(sp[4]), round(sp[5])],
        "release_acquire_one_way": round(sp[6]), "l2_hit_load": round(sp[7])}
    b = torch.from_numpy(gen.rhs(A.n, 1)).to(dev)
    x = torch.empty_like(b)
    P = api._p
    info = api._ws(L.bilu_sptrsv_analysis_bytes(nb), dev)
    ws = api._ws(max(L.bilu_sptrsv_analysis_ws_bytes(nb, nnzb), L.bilu_sptrsv_solve_ws_bytes(nb)),
                 dev)
    strict = (nnzb - nb) // 2
    for lower in (1, 0):
        tag = "L" if lower else "U"
        e0.record()
        api.call("bilu_sptrsv_analysis", nb, nnzb, bs, P(row), P(col), lower, P(info), P(ws),
                 ws.numel(), api._s())
        e1.record()
        e1.synchronize()
        out[f"{tag}_analysis_ms"] = e0.elapsed_time(e1)
        words = info.view(torch.int32).cpu().numpy()
        carve = lambda k: ((k * 4 + 255) // 256) * 64
        o_nlev = 2 * carve(nb + 1) + carve(nb + 2)
        out[f"{tag}_levels"] = int(words[o_nlev])
        out[f"{tag}_recommended"] = "syncfree" if int(words[o_nlev + 2]) == 1 else "level"
        for fn, name in (("bilu_sptrsv_solve_level", "level"),
                         ("bilu_sptrsv_solve_syncfree", "syncfree")):
            def solve():
                api.call(fn, nb, bs, P(row), P(col), P(lu), lower, lower, P(info), P(b), P(x),
                         P(ws), ws.numel(), api._s())
            for _ in range(args.warmup):
                solve()
            e0.record()
            for _ in range(args.steps):
                solve()
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            nbytes = (strict + nb) * (bs * bs * 8 + 4) + (nb + 1) * 4 * 3 + 2 * A.n * 8
            out[f"{tag}_{name}_ms"] = ms
            out[f"{tag}_{name}_GBs"] = nbytes / ms / 1e6
    # GMRES(30) with the exact BILU(0) (two level-scheduled solves per apply)
    # against the FP32 ISAI apply, and the measured switch between them
    Pc = api.Preconditioner(nb, bs, row, col, val, fp32=True, ilu=True, ilu_fp32=True)
    for prec, tag in ((api.BILU_ILU, "ilu"), (api.BILU_ILU_FP32, "ilu_fp32"),
                      (api.BILU_FP32, "isai_fp32")):
        e0.record()
        _, res = Pc.solve(b, x, prec=prec, maxit=args.maxit)
        e1.record()
        e1.synchronize()
        out[f"gmres_{tag}"] = {"s": e0.elapsed_time(e1) / 1e3, "iters": res.iters,
                               "relres": res.relres}
    # ISAI(2): M patterns from pattern(A^2)
    P2 = api.Preconditioner(nb, bs, row, col, val, fp32=True, isai_level=2)
    e0.record()
    _, res = P2.solve(b, x, prec=api.BILU_FP32, maxit=args.maxit)
    e1.record()
    e1.synchronize()
    nnz2 = int(P2.get(2).numel())
    out["gmres_isai2_fp32"] = {"s": e0.elapsed_time(e1) / 1e3, "iters": res.iters,
                               "relres": res.relres, "nnzb_ML": nnz2,
                               "setup_ms": P2.setup_ms["total"]}
    P2.close()
    choice, rate = Pc.select(b, cycles=3)
    out["switch"] = {"choice": {0: "isai_fp64", 1: "isai_fp32", 2: "ilu", 3: "fp32_inner",
                                4: "ilu_fp32"}[choice],
                     "digits_per_s": rate}
    Pc.close()
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "powerlaw":
        run_powerlaw(args)
    elif args.workload == "sptrsv":
        run_sptrsv(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
