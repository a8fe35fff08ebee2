"""GPU parity at the benchmarked sizes: the CUDA grid engine against the
oracle's port of src/boid_simulation_grid.cpp, bit for bit, through the C ABI.

* the uniform-grid workload itself, N = 2^20 in a cube of side 4 (79 device
  cells per axis, 2.0 M x-cells, a single-pass scan over about 1000 tiles):
  its seeded initial state and three updates;
* the same flock after 1000 updates, when it has gathered into dense
  clusters: one update from that state, with the crowded cells on the
  CTA-per-cell kernel and the largest neighbourhoods (more candidates than
  its shared list holds) in id windows;
* the CPU configuration of the reference (N = 16384, F = 1) over its whole
  horizon of 100 updates.
"""
import numpy as np
import pytest

from conftest import assert_bits_equal, make_params, make_sim

pytestmark = pytest.mark.gpu

N_BIG, F_BIG, SEED = 1 << 20, 4.0, 12345


def _port(O, p, pos, vel, steps):
    pos, vel = pos.copy(), vel.copy()
    f = O.GridPort(p, pos).step(pos, vel, steps, forces=True)
    return pos, vel, f


def _candidates_per_cell(pos, G, F):
    """Boids in the 27 device cells around each occupied full-size cell."""
    c = np.minimum((pos.reshape(-1, 3) * (G / F)).astype(np.int64), G - 1)
    occ = np.zeros((G, G, G), np.int64)
    np.add.at(occ, (c[:, 2], c[:, 1], c[:, 0]), 1)
    nb = np.zeros_like(occ)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                nb += np.roll(occ, (dz, dy, dx), axis=(0, 1, 2))
    return occ, nb


@pytest.fixture(scope="module")
def big(boids_lib, oracle_mod):
    O = oracle_mod
    p = make_params(O, N_BIG, F_BIG, O.MARUN2019)
    sim = make_sim(boids_lib, "grid", N_BIG, F_BIG, O.MARUN2019)
    sim.initialization_type = "random_uniform"
    sim.rand_seed = SEED
    yield O, p, sim
    sim.close()


def test_benchmark_workload_init_and_three_updates(big):
    O, p, sim = big
    sim.init()
    pos0, vel0 = O.init_state(p, "random_uniform", True, SEED)
    gp, gv = sim.state()
    assert_bits_equal(gp, pos0, "init positions")
    assert_bits_equal(gv, vel0, "init velocities")
    sim.update(3)
    op, ov, of = _port(O, p, pos0, vel0, 3)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions after 3 updates")
    assert_bits_equal(gv, ov, "velocities after 3 updates")
    assert_bits_equal(sim.forces(), of, "forces of update 3")


def test_benchmark_workload_clustered_update(big):
    """1000 updates on the GPU (replayed graphs), then one update from that
    state on both sides; also the neighbour sets of that state."""
    O, p, sim = big
    sim.init()
    sim.update(1000)
    pos, vel = sim.state()
    pos, vel = pos.reshape(-1).copy(), vel.reshape(-1).copy()
    info = sim.grid_info()
    G = info["dev_cells_per_axis"]
    occ, nb = _candidates_per_cell(pos, G, F_BIG)
    # the state exercises the paths it is here for: crowded cells, and
    # neighbourhoods beyond the dense kernel's 1024-entry list (id windows)
    assert occ.max() >= 64 and nb[occ > 0].max() > 1024, (occ.max(), nb[occ > 0].max())
    gc, gh = sim.neighbor_sets()
    oc, oh = O.neighbor_sets(p, pos, vel)
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh), "neighbour sets"
    assert gc[:, 0].mean() > 20, "the flock has gathered"
    sim.update(1)
    op, ov, of = _port(O, p, pos, vel, 1)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions after update 1001")
    assert_bits_equal(gv, ov, "velocities after update 1001")
    assert_bits_equal(sim.forces(), of, "forces of update 1001")


def test_cpu_configuration_whole_horizon(boids_lib, oracle_mod):
    """N = 16384, F = 1, 100 updates from the seeded initial state, checked
    at every 25th update."""
    O = oracle_mod
    n, field = 16384, 1.0
    p = make_params(O, n, field, O.MARUN2019)
    sim = make_sim(boids_lib, "grid", n, field, O.MARUN2019)
    sim.initialization_type = "random_uniform"
    sim.rand_seed = SEED
    sim.init()
    pos, vel = O.init_state(p, "random_uniform", True, SEED)
    port = O.GridPort(p, pos)
    for t in range(25, 101, 25):
        sim.update(25)
        f = port.step(pos, vel, 25, forces=True)
        gp, gv = sim.state()
        assert_bits_equal(gp, pos, "positions after %d updates" % t)
        assert_bits_equal(gv, vel, "velocities after %d updates" % t)
        assert_bits_equal(sim.forces(), f, "forces of update %d" % t)
    sim.close()
