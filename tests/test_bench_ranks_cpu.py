"""Multi-rank host logic of bench.py without a GPU: the max-over-ranks
reduction behind whole-job times (two gloo ranks), and the reference arm
under torchrun (rank 0 alone runs and prints one line, every rank exits 0)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from tests.conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    q.put((rank, bench.max_over_ranks(10.0 + 5.0 * rank, torch.device("cpu"))))
    torch.distributed.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_process():
    import torch
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, torch.device("cpu")) == 3.5


def test_reference_arm_under_torchrun_two_ranks():
    from fdtd_accelerate_gb300 import build
    build()  # the reference arm times the oracle, built with the library
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--shape", "64,48,40"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["config"]["same_config"] and d["config"]["cells"] == 64 * 48 * 40
