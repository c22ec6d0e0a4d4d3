"""Multi-rank logic of the benchmark on CPU (gloo, world size 2): the path shards by replicas and
instances, so ranks exchange nothing but the final timing reduction."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    local = [120.0, 480.0][rank]
    mx = bench.reduce_max(local, world)
    val = bench.weak_scaling_value(1000.0, world, 4, mx)
    out.put((rank, mx, val))
    dist.destroy_process_group()


def test_reduce_max_and_weak_scaling_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, val in res:
        assert mx == 480.0  # the slowest rank's time
        assert val == pytest.approx(2 * 1000.0 * 4 / 0.48)


def test_reference_arm_under_two_ranks_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-budget", "0.3", "--gpus", "2"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
