"""bench.py's multi-GPU arithmetic (independent replicas, no data-path
collective) with world_size-2 gloo process groups on CPU: the slowest rank's
time and the boid-steps of all ranks; the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    t, u = bench.reduce_over_ranks(dist, 1.0 + rank, 1000.0 * (rank + 1))
    q.put((rank, t, u))
    dist.destroy_process_group()


def test_replica_reduction_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, u in got:
        assert t == 2.0      # the slowest rank
        assert u == 3000.0   # all ranks' boid-steps
    assert bench_value(got[0]) == 1500.0


def bench_value(r):
    return r[2] / r[1]


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, 2.5, 10.0) == (2.5, 10.0)


@pytest.mark.slow
def test_reference_arm_prints_on_rank_zero_only():
    """torchrun --nproc-per-node 2 bench.py --impl reference: one JSON line."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--boids", "4096",
           "--field", "0.63"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and '"impl": "reference"' in lines[0]
    import json
    d = json.loads(lines[0])
    assert d["unit"] == "boid-steps/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["n_gpus"] == 2 and d["steps"] == 1 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["n"] == 4096
