"""The multi-GPU form is replicas only (one independent domain per rank, no
collective on the data path): the bench's host logic across ranks, run as
two gloo processes on the CPU.

Bars: the max-over-ranks reduction gives every rank the slowest rank's
time; under torchrun with two ranks the reference arm prints exactly one
JSON line (rank 0) and both ranks exit 0."""
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


def _rank_main(rank, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    bench.barrier(2, rank)
    got = bench.allreduce_max(1.5 + rank, 2, "reference")
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr(got))
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(free_port(), str(tmp_path)), nprocs=2, join=True)
    vals = [float(open(tmp_path / f"r{r}.txt").read()) for r in range(2)]
    assert vals == [2.5, 2.5]


def test_reference_arm_under_torchrun_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "1", "--workload", "weibel2d_128_o1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
