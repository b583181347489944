"""The N-GPU bench path on CPU: world_size-2 gloo ranks.

The front end has no cross-GPU exchange, so N GPUs run N replicas; what
needs checking is the host side -- the max-over-ranks timing reduction, the
barriers, and that the reference arm prints exactly one line from rank 0
while the other ranks exit cleanly.
"""
import json
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


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.reduce_max(10.0 * (rank + 1), world)
    bench.barrier(world)
    out[rank] = got
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    assert dict(out) == {0: 20.0, 1: 20.0}


def test_reference_arm_under_torchrun():
    """Two ranks launched as the multi-GPU bench is: rank 0 times the CPU
    reference arm and prints one JSON line; rank 1 exits 0 without work."""
    pytest.importorskip("numpy")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
