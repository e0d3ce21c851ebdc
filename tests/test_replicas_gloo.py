"""The N > 1 path of bench.py on CPU with world size 2 over gloo: the path
runs as independent replicas (no data-path collective), joined by a barrier,
timed as the maximum over ranks, and printed by rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init(world)
    assert (r, w) == (rank, world)
    bench.barrier(w)
    # each replica reports its own time; the job's time is the slowest
    out[rank] = bench.max_over_ranks(1.0 + rank, w)
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(2, free_port(), out), nprocs=2, join=True,
                       start_method="spawn")
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--scale", "10", "--steps", "2",
           "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"


def test_printed_lines_are_strict_json():
    """Every line bench.py prints is strict JSON: non-finite floats (a
    comparison on a graph where a quantity is undefined) become null."""
    sys.path.insert(0, ROOT)
    import bench
    line = {"a": float("nan"), "b": [1.5, float("inf"), {"c": -float("inf")}], "d": "x"}
    text = json.dumps(bench.strict(line), allow_nan=False)
    assert json.loads(text) == {"a": None, "b": [1.5, None, {"c": None}], "d": "x"}
