"""The N > 1 path on CPU (gloo, world size 2): replicas reduce their timed
region with a max over ranks and report the whole-job rate; under torchrun
the reference arm of bench.py runs on rank 0 only and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    from pasif_gb300.replicas import job_rate, max_over_ranks
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    slowest = max_over_ranks(1.0 + rank, dist)     # rank r took 1 + r seconds
    out[rank] = (slowest, job_rate(100.0, world, slowest))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = free_port()
        ps = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == out[1] == (2.0, 100.0)    # 2 ranks x 100 units over the slowest 2 s


def test_reference_arm_under_torchrun():
    """`torchrun ... bench.py --impl reference`: rank 0 times the CPU
    restatement and prints the one JSON line; rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0
