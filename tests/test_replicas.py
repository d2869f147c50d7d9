"""The multi-GPU path is replicas only: every rank solves its own copy and the
ranks meet only for the barrier and the max-over-ranks time.  These tests run
that path on the CPU with the gloo backend, world size 2."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _reduce_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mx = bench.max_over_ranks(dist, float(rank + 1) * 10.0)
        sm = bench.sum_over_ranks(dist, float(rank + 1))
        out[rank] = (mx, sm)
    finally:
        dist.destroy_process_group()


def test_max_and_sum_over_two_ranks():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_reduce_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        assert out[0] == out[1] == (20.0, 3.0)


def test_reference_arm_under_torchrun_prints_one_line(zlib, olib):
    """`bench.py --impl reference` launched with two ranks: rank 0 alone times
    the CPU implementation and prints; rank 1 exits 0 without work."""
    import bench
    if not bench.read_reference_inputs("c2"):
        bench.write_reference_inputs()  # build() writes them; a fresh checkout may not have run it
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "c2"]
    env = {**os.environ, "OMP_NUM_THREADS": "2"}
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert "unavailable" not in line, line
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
