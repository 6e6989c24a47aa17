"""Benchmark: block-ILU(0) + ISAI preconditioned GMRES on the 128^3 4-DOF
convection-diffusion system (BSR 4x4, 2,097,152 block rows, 14,581,760
blocks, FP64 matrix), synthetic seeded data.

A step is one solve to 1e-10 relative residual from x0 = 0 with the
mixed-precision path: FP64 flexible GMRES(30) (FP64 residuals,
orthogonalisation and true residual at every restart) whose preconditioned
vectors are --inner steps of FP32 GMRES with the FP32-stored ISAI and the
FP32-stored A (the nested, GMRES-IR form).  The preconditioner setup
(BILU(0) + ISAI on the GPU) runs once before the timed region and is
reported separately, as are the plain FP64 ISAI path (the denominator of
`speedup_mixed_vs_fp64`), the FP32 apply inside flat FGMRES (`fp32_apply`),
the FP32-operator flat variant (`fp32_inner`), other inner lengths
(`nested_inner_scan`) and GMRES with the exact BILU(0) applied by
level-order triangular solves (`exact_ilu`).  `value` is the mean solve time
(s) with the matrix resident in HBM (1.9 GB of values, larger than L2).
`e2e` is the same metric through the C ABI call with host buffers
(bilu_solve_host: H2D of A and b, setup, solve, D2H of x), the first call
of the process.  `roofline` rates the FP32 apply as the inner solver
launches it (two k_bsr_spmv, FP32 vectors in and out) against the measured
copy bandwidth; `traffic` is the DRAM bytes of the same launches from the
committed ncu capture.  `errors` states each mixed-precision result against
the FP64 oracle.  `cpu_baseline` is the oracle's full nested solve on the
host cores (measured, one solve), plus serial (one core) times.
`--impl reference` times the oracle's solve of the same system in every
step.  Secondary lines: --workload sptrsv | powerlaw | batch (give the batch
a step cap, e.g. --maxit 60: its larger systems do not converge).  For ncu:
--workload kernels (the inner solver's products, the FP64 operator product
and the Gram-Schmidt step kernels; --mgs-only for the step kernels alone)
and --profile (setup and solves only; --profile-prec fp64 for the plain
path).

    python bench.py [--steps K] [--warmup W] [--side 128] [--inner 8] [--impl reference]
    torchrun --nproc-per-node N bench.py --gpus N   (N independent replicas)
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
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
    ap.add_argument("--inner", type=int, default=8,
                    help="inner FP32 GMRES steps per outer step of the nested mode")
    ap.add_argument("--workload", default="convdiff",
                    choices=["convdiff", "batch", "powerlaw", "sptrsv", "kernels"],
                    help="convdiff: the headline line; batch / powerlaw / sptrsv: secondary "
                         "lines; kernels: the inner solver's kernels alone, for ncu captures")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-lo", type=int, default=32)
    ap.add_argument("--batch-hi", type=int, default=512)
    ap.add_argument("--batch-rhs", type=int, default=32)
    ap.add_argument("--batch-seed", type=int, default=0)
    ap.add_argument("--batch-mem-gb", type=float, default=96.0)
    ap.add_argument("--batch-schedule", default="persistent", choices=["persistent", "graph"],
                    help="one cooperative launch per Arnoldi step, or a graph of per-phase "
                         "launches")
    ap.add_argument("--pl-nb", type=int, default=500000)
    ap.add_argument("--mgs-only", action="store_true",
                    help="--workload kernels: only the Gram-Schmidt step timings (no system "
                         "setup on the device: small enough for multi-pass ncu captures at 128^3)")
    ap.add_argument("--profile-prec", default="nested", choices=["nested", "fp64"],
                    help="--profile: the solve mode of the warm-up and timed solves")
    ap.add_argument("--profile", action="store_true",
                    help="short run for ncu launch lists: the setup, then --warmup and --steps "
                         "nested solves, nothing else")
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


def measured_traffic(side):
    """DRAM bytes per inner FP32 apply from the committed ncu summary of the
    same launches (profiles/roofline_traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if not os.path.exists(p):
        return None, None
    d = json.load(open(p))
    if d.get("side") != side or d.get("form") != "inner":
        return None, None
    return float(d["dram_bytes_per_apply"]), d.get("source")


def spmv_bytes(nb, bs, nnzb):
    n = nb * bs
    return nnzb * (bs * bs * 8 + 4) + (nb + 1) * 4 + 2 * n * 8


def spmv_bytes_f32(nb, bs, nnzb):
    """FP32 values, FP32 vectors (the inner solver's operator product)."""
    n = nb * bs
    return nnzb * (bs * bs * 4 + 4) + (nb + 1) * 4 + 2 * n * 4


def apply_bytes_inner(nb, bs, nnzL, nnzU):
    """Algorithmic bytes of the FP32 apply as the inner solver runs it:
    FP32 values + column indices of both factors, both row pointers, read
    u (FP32), write and read the intermediate (FP32), write q (FP32)."""
    n = nb * bs
    return (nnzL + nnzU) * (bs * bs * 4 + 4) + 2 * (nb + 1) * 4 + n * 4 * 4


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


# ---------------------------------------------------------------- workload
def convdiff_system(side):
    from isai_kernel_gb300 import gen

    A = gen.convdiff3d(side, bs=4, seed=0)
    return A, gen.rhs(A.n, 0)


def workload_config(args, A):
    """The config dict both arms print (identical by construction)."""
    return {"workload": f"convdiff3d {args.side}^3 bs4 (nb={A.nb}, nnzb={A.nnzb}), "
                        f"FGMRES({args.restart}) to {args.tol:g} from x0 = 0, nested mixed "
                        f"precision: FP64 outer, FP32 inner GMRES({args.inner}) with FP32-stored "
                        f"ISAI and A; setup outside the timed step",
            "nb": A.nb, "nnzb": A.nnzb, "restart": args.restart, "inner": args.inner,
            "tol": args.tol, "parallelism": "single GPU" if args.gpus <= 1 else
            f"replicas x{args.gpus}",
            "l2": "inputs larger than L2 (1.87 GB of FP64 values)"}


# ---------------------------------------------------------------- CPU baseline
def oracle_parts(A):
    from oracle import oracle

    t0 = time.perf_counter()
    S = oracle.isai_setup(A)
    t_setup = time.perf_counter() - t0
    Ab = (A.rowptr, A.colind, A.val)
    L = (S["TrowL"], S["TcolL"], S["McsrL"])
    U = (S["TrowU"], S["TcolU"], S["McsrU"])
    return S, Ab, L, U, t_setup


def cpu_solve(A, b, parts, args, maxit=None):
    """One oracle solve of the headline algorithm (nested mode) from x0 = 0,
    timed on the host: (seconds, x, outer iterations, inner steps, relres)."""
    from oracle import oracle

    _, Ab, L, U, _ = parts
    t0 = time.perf_counter()
    x, it, inner, rr, _, st = oracle.gmres_nested(Ab, L, U, b, inner=args.inner,
                                                  restart=args.restart, tol=args.tol,
                                                  maxit=maxit or args.maxit)
    return time.perf_counter() - t0, x, it, inner, rr, st


def cpu_baseline(A, b, parts, args):
    """The oracle (plain-C restatement of the path, OpenMP over the host
    cores): one full nested solve to 1e-10 of the same system, measured
    (not extrapolated), the setup measured beside it, and the serial (one
    core) BILU(0), ISAI setup, applies and triangular solves."""
    from oracle import oracle

    S, Ab, L, U, t_setup = parts
    t, x, it, inner, rr, st = cpu_solve(A, b, parts, args)
    cores = oracle.num_threads()
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
        del LU
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
    return {"value": t, "unit": "s", "cores": cores, "kind": "port",
            "sample": (f"the oracle's nested solve to {args.tol:g} of the full {args.side}^3 "
                       f"system, measured once ({it} outer / {inner} inner steps, relres "
                       f"{rr:.3g}); its setup measured separately ({t_setup:.2f} s)"),
            "setup_s": t_setup, "iters": it, "inner_steps": inner, "relres": rr, "status": st,
            "serial_1_core": {"bilu0_s": t_f1, "isai_setup_s": t_s1, "apply_fp64_s": t_a64,
                              "apply_fp32_s": t_a32, "sptrsv_L_s": t_l1, "sptrsv_U_s": t_u1},
            "_x": x}


def run_reference(args):
    """The reference arm: the reference has no GPU solver and no Krylov
    method, so its CPU implementation of the path is the oracle (the plain-C
    restatement), run on the host cores with every thread, on the same
    system and algorithm as the GPU arm.  Setup once (reported, outside the
    steps, as on the GPU); every timed step is a full solve to the
    tolerance; warm-up steps run one outer step each (untimed)."""
    rank, world = dist_init(args)
    if rank != 0:
        return
    from oracle import oracle

    A, b = convdiff_system(args.side)
    parts = oracle_parts(A)
    for _ in range(args.warmup):
        cpu_solve(A, b, parts, args, maxit=1)
    times, its = [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        t, x, it, inner, rr, st = cpu_solve(A, b, parts, args)
        times.append(t)
        its.append((it, inner, rr, st))
    wall = time.perf_counter() - t_wall
    v = statistics.mean(times)
    it, inner, rr, st = its[-1]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32",
            "data": "synthetic (seeded 128^3 7-point convection-diffusion, 4 DOF, BSR 4x4)",
            "config": workload_config(args, A),
            "iters": {"outer": it, "inner": inner}, "relres": rr, "status": st,
            "setup_s": parts[4], "step_s": times,
            "cpu_baseline": {"value": v, "unit": "s", "cores": oracle.num_threads(),
                             "kind": "port",
                             "sample": (f"every timed step is the oracle's full nested solve to "
                                        f"{args.tol:g} of the {args.side}^3 system on "
                                        f"{oracle.num_threads()} threads; warm-up steps run "
                                        f"one outer step each; setup {parts[4]:.2f} s once")},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU arm
def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def run_ours(args):
    import torch

    from isai_kernel_gb300 import _lib, api

    rank, world = dist_init(args)
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.lib()
    stream = torch.cuda.current_stream()

    A, b_np = convdiff_system(args.side)
    nb, bs, nnzb, n = A.nb, A.bs, A.nnzb, A.n
    row = torch.from_numpy(A.rowptr).to(dev)
    col = torch.from_numpy(A.colind).to(dev)
    val = torch.from_numpy(A.val).to(dev)
    b = torch.from_numpy(b_np).to(dev)
    torch.cuda.synchronize()

    P = api.Preconditioner(nb, bs, row, col, val, fp32=True, fp32_inner=True, nested=True,
                           inner=args.inner)
    setup_ms = P.setup_ms
    x = torch.empty_like(b)
    NESTED = api.BILU_NESTED

    def solve(prec, out=None):
        return P.solve(b, x if out is None else out, prec=prec, restart=args.restart,
                       tol=args.tol, maxit=args.maxit)

    # the timed mode: the nested solve (a --profile run may take the plain
    # FP64 solve instead, for its launch list)
    MAIN = api.BILU_FP64 if (args.profile and args.profile_prec == "fp64") else NESTED
    for _ in range(args.warmup):
        _, res = solve(MAIN)
    barrier(world)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    l0 = L.bilu_kernel_launches()
    times, iters = [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, res = solve(MAIN)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        iters.append((res.iters, res.inner_steps))
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    launches = L.bilu_kernel_launches() - l0
    res_mixed = res
    x_nested = x.cpu().numpy().copy()
    t_mixed = max_over_ranks(statistics.mean(times), world)
    if args.profile:
        # launch lists: the setup, the warm-up and the timed solves only
        P.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": t_mixed, "unit": "s", "profile": True,
                              "mode": args.profile_prec,
                              "iters": {"outer": res.iters, "inner": res.inner_steps},
                              "gpu_launches": int(launches)}))
        return

    def timed(prec, out=None):
        solve(prec, out)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, r = solve(prec, out)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3, r

    # plain FP64 path: the denominator of the mixed-precision speed-up
    x64 = torch.empty_like(b)
    t_fp64, r64 = timed(api.BILU_FP64, x64)
    # FP32-stored ISAI apply inside flat FP64 FGMRES(30) (FP64 Arnoldi products)
    x32a = torch.empty_like(b)
    t_f32, r32 = timed(api.BILU_FP32, x32a)
    # FP32 ISAI plus FP32-stored A in the Arnoldi products of the flat solver
    t_f32i, r32i = timed(api.BILU_FP32_INNER)
    # the nested mode at other inner lengths (the headline uses --inner)
    inner_scan = {}
    for k in sorted({6, 12, 16, 24} - {args.inner}):
        P.set_inner(k)
        t_k, r_k = timed(NESTED)
        inner_scan[str(k)] = {"s": t_k, "outer": r_k.iters, "inner": r_k.inner_steps,
                              "relres": r_k.relres}
    P.set_inner(args.inner)

    # exact BILU(0) preconditioner (two level-order triangular solves per apply)
    Pi = api.Preconditioner(nb, bs, row, col, val, fp32=False, ilu=True)
    xi = torch.empty_like(b)
    _, ri = Pi.solve(b, xi, prec=api.BILU_ILU, restart=args.restart, tol=args.tol,
                     maxit=args.maxit)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _, ri = Pi.solve(b, xi, prec=api.BILU_ILU, restart=args.restart, tol=args.tol,
                     maxit=args.maxit)
    e1.record(stream)
    e1.synchronize()
    t_ilu = e0.elapsed_time(e1) / 1e3
    ilu_setup = Pi.setup_ms["total"]
    Pi.close()
    del Pi
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

    # kernels timed alone with CUDA events on the launching stream (inputs:
    # 1.1-1.9 GB of factors, larger than L2)
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
    # the apply as the inner solver launches it: two k_bsr_spmv, FP32 in,
    # FP32 intermediate, FP32 out
    b32 = b.float()
    y32 = torch.empty(n, dtype=torch.float32, device=dev)
    q32 = torch.empty(n, dtype=torch.float32, device=dev)
    w32 = torch.empty(n, dtype=torch.float32, device=dev)
    A32 = val.float()

    def apply_inner():
        L.bilu_bcsr_spmv_f32(nb, bs, api._p(Lf[0]), api._p(Lf[1]), api._p(L32), api._p(b32), 1,
                             api._p(y32), 1, api._s())
        L.bilu_bcsr_spmv_f32(nb, bs, api._p(Uf[0]), api._p(Uf[1]), api._p(U32), api._p(y32), 1,
                             api._p(q32), 1, api._s())
    t_apply_in = time_it(apply_inner, reps)
    t_spmvA32 = time_it(lambda: L.bilu_bcsr_spmv_f32(nb, bs, api._p(row), api._p(col),
                                                     api._p(A32), api._p(q32), 1, api._p(w32),
                                                     1, api._s()), reps)
    y = torch.empty_like(b)
    t_spmvA = time_it(lambda: api.bcsr_spmv(nb, bs, row, col, val, b, y), reps)
    B64 = apply_bytes(nb, bs, nnzL, nnzU, 8, 8)
    B32 = apply_bytes(nb, bs, nnzL, nnzU, 4, 4)
    BA = spmv_bytes(nb, bs, nnzb)
    Bin = apply_bytes_inner(nb, bs, nnzL, nnzU)
    BA32 = spmv_bytes_f32(nb, bs, nnzb)
    peak, peak_kind = peaks()
    gbs_in = Bin / t_apply_in / 1e9
    traffic, traffic_src = measured_traffic(args.side)
    rates = (ctypes.c_double * 3)()
    rc = probe_lib().probe_rates(rates)
    assert rc == 0, f"probe_rates returned {rc}"
    dfma_tf = rates[0]
    flops64 = 2.0 * (nnzL + nnzU) * bs * bs
    flopsA = 2.0 * nnzb * bs * bs

    # end to end through the C ABI with pinned host buffers (the nested
    # mode; the first call of the process grows the library's memory pool)
    hrow = torch.from_numpy(A.rowptr).pin_memory()
    hcol = torch.from_numpy(A.colind).pin_memory()
    hval = torch.from_numpy(A.val).pin_memory()
    hb = torch.from_numpy(b_np).pin_memory()
    hx = torch.empty(n, dtype=torch.float64).pin_memory()
    e2e = []
    for _ in range(0 if args.profile else 3):
        it, rr = ctypes.c_int(0), ctypes.c_double(0)
        tm = (ctypes.c_double * 4)()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = L.bilu_solve_host(nb, nnzb, bs, ctypes.c_void_p(hrow.data_ptr()),
                               ctypes.c_void_p(hcol.data_ptr()), ctypes.c_void_p(hval.data_ptr()),
                               ctypes.c_void_p(hb.data_ptr()), ctypes.c_void_p(hx.data_ptr()),
                               NESTED, args.restart, args.tol, args.maxit, ctypes.byref(it),
                               ctypes.byref(rr), tm, ctypes.c_void_p(stream.cuda_stream))
        e2e.append(time.perf_counter() - t0)
        assert st == 0, st
    h2d = A.rowptr.nbytes + A.colind.nbytes + A.val.nbytes + b_np.nbytes
    d2h = n * 8

    # errors against the FP64 oracle, the oracle's solve and the CPU baseline
    cpu, errors = None, None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle

        parts = oracle_parts(A)
        S = parts[0]
        cpu = cpu_baseline(A, b_np, parts, args)
        xo_nested = cpu.pop("_x")
        x64h = x64.cpu().numpy()
        ya = oracle.bcsr_spmv(nb, bs, parts[2][0], parts[2][1], parts[2][2], b_np)
        za = oracle.bcsr_spmv(nb, bs, parts[3][0], parts[3][1], parts[3][2], ya)
        z32 = api.isai_apply(nb, bs, (Lf[0], Lf[1], L32), (Uf[0], Uf[1], U32), b, prec=1)
        # the reference's single-apply check (x_true = 0.7, b = A x_true)
        xt = torch.full((n,), 0.7, dtype=torch.float64, device=dev)
        bk = torch.empty_like(b)
        api.bcsr_spmv(nb, bs, row, col, val, xt, bk)
        kx64 = api.isai_apply(nb, bs, Lf, Uf, bk, prec=0)
        kx32 = api.isai_apply(nb, bs, (Lf[0], Lf[1], L32), (Uf[0], Uf[1], U32), bk, prec=1)
        ka64 = api.compute_rel_errors(nb, bs, row, col, val, bk, xt, kx64)
        ka32 = api.compute_rel_errors(nb, bs, row, col, val, bk, xt, kx32)
        errors = {
            "ML_fp32_vs_oracle_fp64": relerr(L32.cpu().numpy().astype(np.float64), S["McsrL"]),
            "MU_fp32_vs_oracle_fp64": relerr(U32.cpu().numpy().astype(np.float64), S["McsrU"]),
            "apply_fp32_vs_oracle_fp64": relerr(z32.cpu().numpy(), za),
            "apply_fp64_vs_oracle_fp64": relerr(api.isai_apply(nb, bs, Lf, Uf, b, prec=0)
                                                .cpu().numpy(), za),
            "x_nested_vs_fp64_solve": relerr(x_nested, x64h),
            "x_fp32_apply_vs_fp64_solve": relerr(x32a.cpu().numpy(), x64h),
            "x_nested_vs_oracle_nested": relerr(x_nested, xo_nested),
            "single_apply_check_fp64": {"rel_error_x": ka64[0], "rel_residual": ka64[1]},
            "single_apply_check_fp32": {"rel_error_x": ka32[0], "rel_residual": ka32[1]},
            "what": "max |a - b| / max |b|; the FP64 GMRES x equals the oracle's FP64 GMRES x "
                    "within 1e-8 and the FP64 iteration count equals the oracle's (tests)"}
        del parts, S
    P.close()
    if rank != 0:
        return
    it_o, it_i = iters[-1]
    line = {
        "metric": METRIC, "value": t_mixed, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_mixed * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded 128^3 7-point convection-diffusion, 4 DOF, BSR 4x4)",
        "config": workload_config(args, A),
        "iters": {"outer": it_o, "inner": it_i, "fp64": r64.iters, "fp32_apply": r32.iters},
        "restart_cycles": {"mixed": res_mixed.restarts, "fp64": r64.restarts},
        "relres": {"mixed": res_mixed.relres, "fp64": r64.relres},
        "fp64_solve_s": t_fp64, "speedup_mixed_vs_fp64": t_fp64 / t_mixed,
        "fp32_apply": {"s": t_f32, "iters": r32.iters, "relres": r32.relres,
                       "speedup_vs_fp64": t_fp64 / t_f32,
                       "what": "FP32-stored ISAI apply inside flat FP64 FGMRES(30) "
                               "(FP64 Arnoldi products and orthogonalisation)"},
        "fp32_inner": {"s": t_f32i, "iters": r32i.iters, "relres": r32i.relres,
                       "speedup_vs_fp64": t_fp64 / t_f32i,
                       "what": "flat FGMRES(30) with FP32 ISAI and FP32-stored A in the Arnoldi "
                               "products; FP64 orthogonalisation, true residual and restarts"},
        "nested_inner_scan": inner_scan,
        "exact_ilu": {"s": t_ilu, "iters": ri.iters, "relres": ri.relres,
                      "setup_ms": ilu_setup, "speedup_vs_fp64_isai": t_fp64 / t_ilu,
                      "what": "FP64 FGMRES(30) with the exact BILU(0) applied by two "
                              "level-order block triangular solves"},
        "exact_ilu_fp32": {"s": t_iluf, "iters": rf.iters, "relres": rf.relres,
                           "setup_ms": iluf_setup, "speedup_vs_fp64_isai": t_fp64 / t_iluf,
                           "what": "FP64 FGMRES(30) with the exact BILU(0) applied in FP32 "
                                   "(FP32 copy of the factor, FP32 level-order solves)"},
        "setup_ms": setup_ms,
        "apply": {"fp32_s": t_apply32, "fp64_s": t_apply64, "fp32_GBs": B32 / t_apply32 / 1e9,
                  "inner_s": t_apply_in, "inner_GBs": gbs_in, "bytes_inner": Bin,
                  "fp64_GBs": B64 / t_apply64 / 1e9, "bytes_fp32": B32, "bytes_fp64": B64,
                  "A_spmv_s": t_spmvA, "A_spmv_GBs": BA / t_spmvA / 1e9,
                  "A32_spmv_s": t_spmvA32, "A32_spmv_GBs": BA32 / t_spmvA32 / 1e9},
        "roofline": {"bound": "hbm", "achieved": gbs_in, "peak": peak, "unit": "GB/s",
                     "frac": gbs_in / peak, "traffic": traffic,
                     "algorithmic_bytes": Bin, "duration_s": t_apply_in,
                     "kernel": "FP32-stored ISAI apply as the inner solver runs it "
                               "(k_bsr_spmv x2: M_L then M_U, FP32 vectors in and out)",
                     "traffic_source": traffic_src,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "fp64_compute_roofline": {
            "dfma_tflops": dfma_tf, "dmma_tflops": rates[1], "ffma_tflops": rates[2],
            "apply_fp64_frac_of_dfma": flops64 / t_apply64 / 1e12 / dfma_tf,
            "A_spmv_frac_of_dfma": flopsA / t_spmvA / 1e12 / dfma_tf,
            "apply_fp64_bound_s": max(flops64 / (dfma_tf * 1e12), B64 / (peak * 1e9)),
            "A_spmv_bound_s": max(flopsA / (dfma_tf * 1e12), BA / (peak * 1e9))},
        "errors": errors,
        "cpu_baseline": cpu,
        "e2e": {"value": max_over_ranks(e2e[0], world) if e2e else None, "unit": "s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "first_call": e2e[0] if e2e else None,
                "repeat_calls": e2e[1:],
                "what": "bilu_solve_host from pinned host buffers: H2D of A and b, setup, "
                        "nested solve, D2H of x; value = the first call of the process"},
        "gpu_launches": int(launches),
        "clocks": clk, "wall_s": wall,
    }
    print(json.dumps(line))


def run_batch(args):
    """Secondary line: 256 seeded 2D 5-point 4-DOF systems, grid sides
    U{32..512} (seed s for system s), 32 uniform right-hand sides each, FP32
    ISAI apply inside FP64 FGMRES(30), all systems in one block-diagonal
    setup, every Arnoldi step one cooperative launch over all (system, tile)
    work of the wave; --maxit caps the Arnoldi steps per wave.  Systems of
    this generator from a side of about 128 on are indefinite and restarted
    GMRES stagnates on them, so the line reports the converged fraction by
    grid side alongside the throughput."""
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
    bt.set_schedule(args.batch_schedule == "persistent")
    Bd = torch.from_numpy(B).cuda()
    X, iters, relres, stats = bt.solve(Bd, restart=args.restart, tol=args.tol, maxit=args.maxit,
                                       mem_budget=int(args.batch_mem_gb * (1 << 30)))
    cfg, tune_ms = bt.tuning()
    conv = float(np.mean(relres <= args.tol))
    by_side = []
    for lo, hi in ((32, 64), (65, 96), (97, 128), (129, 256), (257, 512)):
        sel = (sides >= lo) & (sides <= hi)
        if sel.any():
            ok = relres[sel] <= args.tol
            by_side.append({"sides": f"{lo}..{hi}", "systems": int(sel.sum()),
                            "converged_fraction": float(ok.mean()),
                            "median_iters_converged": float(np.median(iters[sel][ok]))
                            if ok.any() else None})
    line = {"workload": f"batch {args.batch_count} x laplace2d U{{{args.batch_lo}..{args.batch_hi}}}"
                        f" bs4, {k} rhs, FGMRES({args.restart}) FP32 ISAI, maxit {args.maxit}",
            "systems": args.batch_count, "rhs": k, "block_rows": bt.nb,
            "setup_s": t_setup, "solve_s": stats[3] / 1e3, "waves": int(stats[0]),
            "graph_launches": int(stats[1]), "pair_steps": int(stats[2]),
            "pair_steps_per_s": stats[2] / (stats[3] / 1e3),
            "converged_fraction": conv, "median_iters": float(np.median(iters)),
            "by_side": by_side,
            "schedule": ("one cooperative launch per Arnoldi step"
                         if args.batch_schedule == "persistent" else
                         "a replayed graph of per-phase launches per Arnoldi step"),
            "ms_per_step": stats[3] / max(1, int(stats[1])),
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
    # the first setup grows the library's memory pool (the CUDA driver maps
    # ~20 GB, at a cost that differs from machine to machine); the second one, after
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
    # ISAI(2) and ISAI(3): M patterns from pattern(A^k); the flat FP64 and
    # FP32-apply solves and the nested mode on each
    for level in (2, 3):
        try:
            Pk = api.Preconditioner(nb, bs, row, col, val, fp32=True, nested=True,
                                    isai_level=level)
        except RuntimeError as exc:  # a pattern row beyond the symbolic product's limit
            out[f"isai{level}"] = {"unavailable": str(exc)}
            continue
        rec = {"nnzb_ML": int(Pk.get(2).numel()), "nnzb_MU": int(Pk.get(5).numel()),
               "setup_ms": Pk.setup_ms["total"]}
        for prec, tag in ((api.BILU_FP64, "fp64"), (api.BILU_FP32, "fp32_apply"),
                          (api.BILU_NESTED, "nested")):
            e0.record()
            _, res = Pk.solve(b, x, prec=prec, maxit=args.maxit)
            e1.record()
            e1.synchronize()
            rec[tag] = {"s": e0.elapsed_time(e1) / 1e3, "iters": res.iters,
                        "relres": res.relres}
            if prec == api.BILU_NESTED:
                rec[tag]["inner"] = res.inner_steps
        Pk.close()
        out[f"isai{level}"] = rec
    choice, rate = Pc.select(b, cycles=3)
    out["switch"] = {"choice": {0: "isai_fp64", 1: "isai_fp32", 2: "ilu", 3: "fp32_inner",
                                4: "ilu_fp32"}[choice],
                     "digits_per_s": rate}
    Pc.close()
    print(json.dumps(out))


def run_kernels(args):
    """For ncu captures: the setup of the --side^3 system, then --steps
    rounds of the inner solver's products as it launches them: M_L u and
    M_U t (k_bsr_spmv, FP32 values and vectors) and A q (FP32-stored A),
    each round in this order (three k_bsr_spmv launches per round), then
    --steps FP64 operator products (k_bsr_spmv, FP64 values and vectors),
    then the Gram-Schmidt step timings.  --mgs-only: the step timings alone,
    on vectors of the system's length."""
    import torch

    from isai_kernel_gb300 import _lib, api

    L = _lib.lib()
    dev = torch.device("cuda", 0)
    p_ = api._p
    if args.mgs_only:
        n = 4 * args.side ** 3  # 4 DOF per grid point
    else:
        A, b_np = convdiff_system(args.side)
        nb, bs, n = A.nb, A.bs, A.n
        row, col, val = (torch.from_numpy(a).to(dev) for a in (A.rowptr, A.colind, A.val))
        P = api.Preconditioner(nb, bs, row, col, val, fp32=True, nested=True)
        _, Lf, Uf = P.factors()
        L32, U32 = P.get(7), P.get(8)
        A32 = val.float()
        u = torch.from_numpy(b_np).to(dev).float()
        t, q, w = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
        for _ in range(args.steps):
            L.bilu_bcsr_spmv_f32(nb, bs, p_(Lf[0]), p_(Lf[1]), p_(L32), p_(u), 1, p_(t), 1,
                                 api._s())
            L.bilu_bcsr_spmv_f32(nb, bs, p_(Uf[0]), p_(Uf[1]), p_(U32), p_(t), 1, p_(q), 1,
                                 api._s())
            L.bilu_bcsr_spmv_f32(nb, bs, p_(row), p_(col), p_(A32), p_(q), 1, p_(w), 1,
                                 api._s())
        # then --steps FP64 operator products (the outer solver's A z)
        z64, y64 = u.double(), torch.empty(n, dtype=torch.float64, device=dev)
        for _ in range(args.steps):
            L.bilu_bcsr_spmv(nb, bs, p_(row), p_(col), p_(val), p_(z64), p_(y64), api._s())
        torch.cuda.synchronize()
        P.close()
        del P, A32, row, col, val, t, q, w, u, z64, y64
    # one orthogonalisation step (j = 15: 17 fused sweeps) on basis vectors
    # of the system's length, FP64 and FP32, CUDA events after a warm-up
    out = {"workload": f"kernels convdiff3d {args.side}^3", "rounds": args.steps}
    ldv = (n + 31) // 32 * 32
    wsb = L.bilu_debug_mgs_step_ws_bytes()
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    j = 15
    rates = (ctypes.c_double * 3)()
    probe_lib().probe_rates(rates)
    for fp32, dt in ((0, torch.float64), (1, torch.float32)):
        g = torch.Generator(device=dev).manual_seed(1)
        # basis vectors of about unit norm (the sweeps then neither grow nor
        # overflow w)
        V = torch.randn((j + 1) * ldv, dtype=dt, device=dev, generator=g) / math.sqrt(n)
        w0 = torch.randn(ldv, dtype=dt, device=dev, generator=g)
        w = torch.empty_like(w0)
        h = torch.empty(j + 2, dtype=torch.float64, device=dev)
        vn = torch.empty_like(w0)
        times = []
        for rep in range(args.steps + 1):
            w.copy_(w0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            rc = L.bilu_debug_mgs_step(n, fp32, p_(V), ldv, j, p_(w), p_(h), p_(vn), p_(ws), wsb,
                                       api._s())
            e1.record()
            e1.synchronize()
            assert rc == 0, rc
            if rep:
                times.append(e0.elapsed_time(e1) * 1e3)
        us = statistics.mean(times)
        sweeps = j + 2
        key = "mgs_step_fp32" if fp32 else "mgs_step_fp64"
        out[key] = {"us_per_step": us, "sweeps": sweeps, "us_per_sweep": us / sweeps}
        if not fp32:
            # two DFMAs per element and sweep (update and dot product)
            floor = 2 * n * 2 / (rates[0] * 1e12) * 1e6
            out[key]["dfma_floor_us_per_sweep"] = floor
            out[key]["frac_of_dfma_floor"] = floor / (us / sweeps)
        else:
            # one basis vector from DRAM per sweep (w and v_i stay in the L2)
            peak, _ = peaks()
            out[key]["hbm_floor_us_per_sweep"] = n * 4 / (peak * 1e9) * 1e6
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
    elif args.workload == "kernels":
        run_kernels(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
