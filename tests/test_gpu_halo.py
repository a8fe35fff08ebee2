"""The domain-decomposed flock's GPU path: boids_set_population (a handle
created for N boids updating a smaller population) against a handle made
for that population, and two ranks (two processes sharing the GPU, gloo
exchange on the host) against one handle holding the whole flock, bit for
bit."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT, assert_bits_equal, make_sim

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MARUN2019 = dict(sep=(0.01, 0.5, 0.002), ali=(0.05, 0.3333333333333333, 0.06),
                 coh=(0.05, 0.5, 0.008), vmax=0.005, vmin=0.001)


def test_smaller_population_equals_its_own_handle(boids_lib, oracle_mod):
    O = oracle_mod
    n, field, sub = 20000, 1.1, 7000
    big = make_sim(boids_lib, "grid", n, field, O.MARUN2019)
    small = make_sim(boids_lib, "grid", sub, field, O.MARUN2019)
    big.init()
    pos, vel = big.state()
    ids = np.sort(np.random.default_rng(5).choice(n, sub, replace=False))
    p, v = pos[ids].copy(), vel[ids].copy()
    big.set_population(p, v)
    small.set_state(p, v)
    for _ in range(3):
        big.update(5)
        small.update(5)
        gp, gv = big.state()
        sp, sv = small.state()
        assert gp.shape == (sub, 3)
        assert_bits_equal(gp, sp, "positions")
        assert_bits_equal(gv, sv, "velocities")
        assert_bits_equal(big.forces(), small.forces(), "forces")
    big.set_state(pos, vel)   # the whole population again
    assert big.state()[0].shape == (n, 3)
    big.update(2)
    big.close()
    small.close()


def _collect(q, procs, limit=300):
    """Rank 0's result, or a failure as soon as a rank has exited with an
    error (its result would never come)."""
    import queue
    import time
    t0 = time.time()
    while time.time() - t0 < limit:
        try:
            return q.get(timeout=2)
        except queue.Empty:
            if any(p.exitcode not in (None, 0) for p in procs):
                for p in procs:
                    p.join(30)
                raise AssertionError("a rank failed: exit codes %r" % [p.exitcode for p in procs])
    raise AssertionError("no result from rank 0 within %d s" % limit)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, field, steps, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        from boidssimulatormpi_gb300.halo import HaloFlock
        m = MARUN2019
        hf = HaloFlock(n, field, m["sep"], m["ali"], m["coh"], m["vmax"], m["vmin"],
                       group=dist.group.WORLD, topology=(1, 1, world), device=0)
        hf.init("random_uniform", 12345)
        hf.update(steps)
        gp, gv = hf.gather()
        hf.engine.close()
        if rank == 0:
            q.put((gp.tobytes(), gv.tobytes()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_equal_one_handle(boids_lib):
    import torch.multiprocessing as mp
    n, field, steps = 20000, 1.1, 40
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, field, steps, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = _collect(q, procs)
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    m = MARUN2019
    sim = boids_lib.BoidSimulation("grid")
    sim.setup(n, field, *m["sep"], *m["ali"], *m["coh"], m["vmax"], m["vmin"], "random_uniform", 12345)
    sim.init()
    sim.update(steps)
    op, ov = sim.state()
    sim.close()
    assert_bits_equal(np.frombuffer(got[0], np.float32), op, "positions")
    assert_bits_equal(np.frombuffer(got[1], np.float32), ov, "velocities")
