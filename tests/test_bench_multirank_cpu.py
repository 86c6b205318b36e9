"""The bench's multi-process path on CPU: ranks are replicas, so the only
cross-rank step is the maximum of the step times (bench.max_over_ranks),
checked here over world_size-2 gloo ranks; and the reference arm under
torchrun prints one line from rank 0 while the other rank exits cleanly."""
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


def _rank(rank, world, port, out):
    import torch

    sys.path.insert(0, ROOT)
    import bench

    torch.distributed.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(torch, [1.0 + rank, 10.0 - rank, 0.5], "cpu")
        with open(os.path.join(out, f"r{rank}.json"), "w") as f:
            json.dump(got, f)
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        with open(tmp_path / f"r{r}.json") as f:
            assert json.load(f) == [2.0, 10.0, 0.5]
    # one process: the values come back unchanged
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(torch, [3.0, 4.0], "cpu") == [3.0, 4.0]


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--chi", "6"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["config"]["workload"] == "mera_ternary_chi6" and d["e2e"]["h2d_bytes_per_step"] == 0
