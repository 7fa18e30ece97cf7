"""bench.py's multi-rank path on the CPU (gloo, world size 2): the max-over-ranks
timing and the barrier, and the reference arm under torchrun (rank 0 alone
runs and prints one JSON line; the other rank exits 0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    w, r, _ = bench.dist_setup(argparse.Namespace(impl="reference"))
    m = bench.reduce_max(1.5 + r, w)
    bench.barrier(w)
    with open(os.path.join(out_dir, "rank%d.json" % r), "w") as f:
        json.dump({"world": w, "rank": r, "max": m}, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_reduce_max_and_barrier_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for r in range(2):
        d = json.load(open(tmp_path / ("rank%d.json" % r)))
        assert d == {"world": 2, "rank": r, "max": 2.5}


def test_reference_arm_under_torchrun():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--workload", "uniform16", "--steps", "2",
           "--warmup", "3"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(l) for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
