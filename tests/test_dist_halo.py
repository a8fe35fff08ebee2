"""The domain-decomposed flock (boidssimulatormpi_gb300/halo.py, the
counterpart of BoidSimulationMultiNode, src/boid_simulation_mpi.cpp) on CPU:
gloo process groups of 2, 3, 4 and 8 ranks, each rank's local update done by
the oracle's port of src/boid_simulation_grid.cpp; the gathered flock equals
one port holding the whole flock, bit for bit (30 updates of 3000 boids;
and the reference's test/compare_mpi.sh, which compares 8 MPI ranks with the
serial engine: N=1000, T=100, settings/test.ini).  Also the block and
margin arithmetic against a direct check."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")

MARUN2019 = dict(sep=(0.01, 0.5, 0.002), ali=(0.05, 0.3333333333333333, 0.06),
                 coh=(0.05, 0.5, 0.008), vmax=0.005, vmin=0.001)
TEST_INI = dict(sep=(0.1, 0.9, 0.0001), ali=(0.1, 0.7, 0.1), coh=(0.1, 0.8, 0.1), vmax=0.003, vmin=0.001)


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


class PortEngine:
    """The oracle's port of the grid engine behind the engine interface
    HaloFlock uses (test infrastructure: the local update on CPU)."""
    record_forces = True

    def __init__(self, O, field, prm):
        self.O, self.F, self.prm = O, field, prm

    def set_population(self, pos, vel):
        self.pos = np.ascontiguousarray(pos, np.float32).reshape(-1).copy()
        self.vel = np.ascontiguousarray(vel, np.float32).reshape(-1).copy()

    def update(self, steps):
        m = self.prm
        p = self.O.params(self.pos.size // 3, self.F, m["sep"], m["ali"], m["coh"], m["vmax"], m["vmin"])
        self.f = self.O.GridPort(p, self.pos).step(self.pos, self.vel, steps, forces=True)

    def state(self):
        return self.pos.reshape(-1, 3), self.vel.reshape(-1, 3)

    def forces(self):
        return np.asarray(self.f, np.float32).reshape(-1, 9)


def _start(n, field, seed, gathered, m=MARUN2019):
    sys.path.insert(0, ROOT)
    import oracle as O
    p = O.params(n, field, m["sep"], m["ali"], m["coh"], m["vmax"], m["vmin"])
    if gathered == "test":  # the reference's `test` placement, never seeded (boidsim)
        pos, vel = O.init_state(p, "test", False, seed)
        return O, p, pos, vel
    pos, vel = O.init_state(p, "random_uniform", True, seed)
    if gathered:  # boids bunched around points on block edges and corners
        rng = np.random.default_rng(seed)
        centres = np.array([[0.5, 0.5, 0.5], [0.0, 0.5, 0.02], [0.25, 0.99, 0.5], [0.5, 0.0, 0.0]]) * field
        q = (centres[rng.integers(len(centres), size=n)] + rng.normal(0, 0.03 * field, (n, 3))) % field
        pos = q.astype(np.float32).reshape(-1)
        pos[pos >= np.float32(field)] = 0.0
    return O, p, pos, vel


def _worker(rank, world, port, topology, n, field, steps, gathered, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = TEST_INI if gathered == "test" else MARUN2019
        O, p, pos, vel = _start(n, field, 7, gathered, m)
        from boidssimulatormpi_gb300.halo import HaloFlock
        hf = HaloFlock(n, field, m["sep"], m["ali"], m["coh"], m["vmax"], m["vmin"],
                       engine=PortEngine(O, field, m), group=dist.group.WORLD, topology=topology)
        hf.set_global_state(pos, vel)
        local0 = len(hf.ids)
        hf.update(steps)
        gp, gv = hf.gather()
        gf = hf.gather_forces()
        if rank == 0:
            q.put((gp.tobytes(), gv.tobytes(), local0, gf.tobytes()))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,topology,gathered,n,steps", [
    (2, (1, 1, 2), False, 3000, 30), (3, (1, 1, 3), True, 3000, 30), (4, (1, 2, 2), True, 3000, 30),
    # test/compare_mpi.sh: 8 ranks, N=1000, T=100, settings/test.ini (test placement)
    (8, (2, 2, 2), "test", 1000, 100)])
def test_decomposed_flock_equals_one_engine(world, topology, gathered, n, steps):
    import torch.multiprocessing as mp
    field = 1.0
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, topology, n, field, steps, gathered, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got = _collect(q, procs)
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    gp = np.frombuffer(got[0], np.float32).reshape(-1)
    gv = np.frombuffer(got[1], np.float32).reshape(-1)
    assert 0 < got[2] < n  # rank 0 holds a part of the flock
    O, p, pos, vel = _start(n, field, 7, gathered, TEST_INI if gathered == "test" else MARUN2019)
    op, ov = pos.copy(), vel.copy()
    of = np.asarray(O.GridPort(p, op).step(op, ov, steps, forces=True), np.float32).reshape(-1)
    gf = np.frombuffer(got[3], np.float32)
    assert np.array_equal(gp.view(np.uint32), op.view(np.uint32)), "positions"
    assert np.array_equal(gv.view(np.uint32), ov.view(np.uint32)), "velocities"
    assert np.array_equal(gf.view(np.uint32), of.view(np.uint32)), "forces of the last update"


def test_dims_create_balances():
    sys.path.insert(0, ROOT)
    from boidssimulatormpi_gb300.halo import dims_create
    assert dims_create(1) == (1, 1, 1)
    assert dims_create(2) == (1, 1, 2)
    assert dims_create(4) == (1, 2, 2)
    assert dims_create(6) == (1, 2, 3)
    assert dims_create(8) == (2, 2, 2)
    assert dims_create(12) == (2, 2, 3)


@pytest.mark.parametrize("topology", [(1, 1, 2), (2, 2, 2), (1, 3, 4)])
def test_destinations_are_the_regions_that_hold_a_boid(topology):
    """Every rank whose block, widened by the margin on each side (across
    the periodic faces too), contains the boid, and no other."""
    sys.path.insert(0, ROOT)
    from boidssimulatormpi_gb300.halo import Decomposition
    F, margin = 1.3, 0.07
    dec = Decomposition(F, topology, margin)
    rng = np.random.default_rng(3)
    pos = (rng.random((4000, 3)) * F).astype(np.float32)
    pos[:50] = np.float32(0.0)
    pos[50:100, 2] = np.float32(F)
    bi, br = dec.destinations(pos)
    got = set(zip(bi.tolist(), br.tolist()))
    d = np.asarray(topology)
    w = F / d
    want = set()
    for r in range(dec.size):
        b = dec.block_of_rank(r)
        inside = np.ones(len(pos), bool)
        for a in range(3):
            if d[a] == 1:
                continue
            x = pos[:, a].astype(np.float64)
            lo, hi = b[a] * w[a], (b[a] + 1) * w[a]
            # distance outside [lo, hi) along the axis, periodic
            dist_lo = np.minimum((lo - x) % F, F)   # how far below lo
            dist_hi = (x - hi) % F                   # how far at or above hi
            ins = (x >= lo) & (x < hi) | ((b[a] == d[a] - 1) & (x >= F))
            near = (dist_lo <= margin) & ~ins | (dist_hi < margin) & ~ins
            inside &= ins | near
        want |= {(i, r) for i in np.nonzero(inside)[0].tolist()}
    # the owner is always among the destinations
    own = dec.owners(pos)
    assert all((i, int(own[i])) in got for i in range(len(pos)))
    assert got == want


def test_blocks_thinner_than_twice_the_margin_are_refused():
    sys.path.insert(0, ROOT)
    from boidssimulatormpi_gb300.halo import Decomposition
    Decomposition(1.0, (1, 1, 5), 0.1)          # 0.2 thick: enough
    with pytest.raises(ValueError, match="thinner"):
        Decomposition(1.0, (1, 1, 6), 0.1)      # 0.167 thick
    with pytest.raises(ValueError, match="positive"):
        Decomposition(1.0, (1, 0, 2), 0.1)


def test_single_rank_keeps_every_boid():
    """Without a process group the flock is one block: every boid is owned
    and nothing is exchanged; the updates equal the port's."""
    sys.path.insert(0, ROOT)
    from boidssimulatormpi_gb300.halo import HaloFlock
    n, field = 500, 0.8
    O, p, pos, vel = _start(n, field, 11, False)
    m = MARUN2019
    hf = HaloFlock(n, field, m["sep"], m["ali"], m["coh"], m["vmax"], m["vmin"],
                   engine=PortEngine(O, field, m))
    hf.set_global_state(pos, vel)
    assert len(hf.ids) == n
    hf.update(5)
    gp, gv = hf.gather()
    op, ov = pos.copy(), vel.copy()
    O.GridPort(p, op).step(op, ov, 5, forces=False)
    assert np.array_equal(gp.reshape(-1).view(np.uint32), op.view(np.uint32))
    assert np.array_equal(gv.reshape(-1).view(np.uint32), ov.view(np.uint32))
