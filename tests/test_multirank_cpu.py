"""The N > 1 host path of bench.py on CPU (gloo, world size 2): every rank
times its own replica and the reported time is the maximum over ranks; under
torchrun only rank 0 prints the JSON line and every rank exits 0.  (The GPU
path shards nothing: BILU(0) and the triangular solves are dependency chains,
so N GPUs run N independent replicas.)"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        gpus = world

    r, w = bench.dist_init(Args())
    assert (r, w) == (rank, world)
    bench.barrier(w)
    v = bench.max_over_ranks(1.5 + rank, w)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(v))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(2)]
    assert vals == [2.5, 2.5]


def test_reference_arm_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--side", "10", "--steps", "2", "--warmup", "1"]
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                         env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    # every timed step is a full solve of the same workload the GPU arm runs
    assert d["relres"] <= 1e-10 and d["status"] == 0 and len(d["step_s"]) == 2
    assert d["iters"]["inner"] == d["iters"]["outer"] * d["config"]["inner"]
    assert d["config"]["workload"].startswith("convdiff3d 10^3 bs4")


def test_bench_options_parse(monkeypatch):
    """The measurement modes the docstring and the profiles name parse, with
    the defaults the headline line uses."""
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert (a.gpus, a.steps, a.warmup, a.side, a.inner, a.impl) == (1, 5, 3, 128, 8, "ours")
    assert a.workload == "convdiff" and not a.profile and not a.mgs_only
    assert a.profile_prec == "nested"
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "kernels", "--side", "96",
                                      "--mgs-only", "--profile", "--profile-prec", "fp64",
                                      "--maxit", "60", "--impl", "reference"])
    a = bench.parse()
    assert (a.workload, a.side, a.mgs_only, a.profile, a.profile_prec, a.maxit, a.impl) == (
        "kernels", 96, True, True, "fp64", 60, "reference")
