"""The N>1 path of bench.py on the CPU (gloo, world size 2): the path does not
shard on one box, so N ranks run N independent replicas with a barrier and a
max-over-ranks of the timings, and the reference arm runs on rank 0 alone."""

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


def _dist_child(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench

    d = bench.Dist()
    d.barrier()
    v = d.max(float(10 * rank + 1))
    d.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": d.rank, "world": d.world, "max": v}, f)
    d.close()


def test_dist_barrier_and_max_over_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = free_port()
    mp.spawn(_dist_child, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        got = json.load(open(tmp_path / f"rank{r}.json"))
        assert got == {"rank": r, "world": 2, "max": 11.0}


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--grid", "16", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
