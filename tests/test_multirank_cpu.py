"""Two-rank runs on the CPU (gloo): the multi-process paths of bench.py without a GPU.

The library runs one process per GPU with replicas only (rows of C shard with no exchange
but a scan of per-shard counts, and the runs here have one GPU each), so the
multi-rank logic under test is the bench's: a torchrun launch whose reference arm runs on
rank 0 alone, and the max-over-ranks reduction of a per-rank time.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", *args]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


@pytest.fixture(scope="module")
def oracle_built():
    import oracle

    oracle.build()


def test_reference_arm_two_ranks(oracle_built):
    """`bench.py --impl reference` under torchrun with two ranks: rank 0 times the CPU
    baseline and prints one JSON line, rank 1 exits 0 without work."""
    r = _torchrun(["--impl", "reference", "--workload", "laplacian", "--gpus", "2", "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["unit"] == "GFLOPS" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


@pytest.mark.parametrize("workload", ["batched", "backward"])
def test_reference_arm_two_ranks_unavailable_form(workload):
    """The batched and backward workloads have no reference implementation: rank 0 prints
    the `unavailable` line, without touching a GPU, and both ranks exit 0."""
    r = _torchrun(["--impl", "reference", "--workload", workload, "--gpus", "2", "--steps", "1", "--warmup", "3"])
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and "unavailable" in lines[0]


def _max_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        q.put((rank, bench.max_over_ranks(1.5 + rank, world, torch.device("cpu"))))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    """The bench reports the slowest rank's time: every rank sees the maximum."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got == {0: 2.5, 1: 2.5}
