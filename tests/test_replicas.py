"""The bench's replica plumbing on N > 1 processes, on CPU with gloo (no GPU): the barrier and the
max-over-ranks timing the driver's torchrun launch uses, and the reference arm's rule that rank 0 alone
runs and prints while the other ranks exit without work."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_setup(argparse.Namespace(impl="reference"))
    bench.barrier(w)
    most = bench.max_over_ranks(float(10 * (r + 1)), w)
    with open(f"{out}.{r}", "w") as f:
        json.dump({"rank": r, "world": w, "local": local, "max": most}, f)
    dist.destroy_process_group()


def test_max_over_ranks_on_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    out = str(tmp_path / "rank")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = [json.load(open(f"{out}.{r}")) for r in range(2)]
    assert [g["rank"] for g in got] == [0, 1] and all(g["world"] == 2 for g in got)
    assert all(g["max"] == 20.0 for g in got)


def test_reference_arm_under_torchrun(oracle_lib, lib):
    """`bench.py --impl reference` launched as two ranks: rank 0 times the CPU path and prints one line,
    rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    run = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [json.loads(x) for x in run.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"


def test_reference_arm_loads_no_cuda_library(oracle_lib):
    """The reference arm's inputs and trace come from the oracle's library alone: after a run, the process
    has mapped liboracle.so and not the CUDA library (nor torch's CUDA runtime)."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']; "
            "runpy.run_path('bench.py', run_name='__main__'); maps = open('/proc/self/maps').read(); "
            "print('MAPS', 'libartful_cuda' in maps, 'liboracle' in maps, 'libcudart' in maps)")
    run = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]
    maps = [x for x in run.stdout.splitlines() if x.startswith("MAPS")]
    assert maps == ["MAPS False True False"], run.stdout[-2000:]
    line = json.loads([x for x in run.stdout.splitlines() if x.startswith("{")][0])
    assert line["config"]["workload"].startswith("kerr-hole 1920x1080")
    assert "whole 1920x1080 frame" in line["cpu_baseline"]["sample"]
