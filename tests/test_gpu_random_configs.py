"""GPU parity on seeded random configurations: flock sizes, densities, rule
radii, view angles (some all-round), weights, speed limits and dense-cell
thresholds drawn at random, each run bit for bit against the oracle's port
of src/boid_simulation_grid.cpp (grid engine) or of src/boid_simulation.cpp
(all-pairs engine, also from states partly outside the field).

The draws are fixed by the seeds below, so every run checks the same cases.
"""
import numpy as np
import pytest

from conftest import assert_bits_equal, make_params, make_sim

pytestmark = pytest.mark.gpu

STEPS = 8
# dense-cell thresholds: the default, everything to the CTA-per-cell kernel
# that can go there, nothing there, and mixed ones
TUNINGS = [(16, 4, 192, 96), (1, 1, 1, 1), (1 << 30, 1 << 30, 1 << 30, 1 << 30), (4, 2, 64, 32), (24, 8, 256, 160)]


def draw(seed):
    """One random configuration: (n, field, settings, tuning)."""
    rng = np.random.default_rng(seed)
    n = int(round(2 ** rng.uniform(7, 15)))
    density = 2 ** rng.uniform(11, 17)            # boids per unit volume
    field = float((n / density) ** (1.0 / 3.0))
    scale = density ** (-1.0 / 3.0)               # mean spacing
    r_far = float(min(field / 6.5, scale * rng.uniform(1.5, 4.0)))  # at least 3 grid cells per axis
    sep = (float(r_far * rng.uniform(0.1, 0.6)), float(rng.choice([rng.uniform(0.15, 0.95), 1.0])),
           float(10 ** rng.uniform(-4, -1.5)))
    ali = (float(r_far * rng.uniform(0.6, 1.0)), float(rng.choice([rng.uniform(0.15, 0.95), 1.0])),
           float(10 ** rng.uniform(-2.5, -0.7)))
    coh = (r_far, float(rng.choice([rng.uniform(0.15, 0.95), 1.0])), float(10 ** rng.uniform(-3, -1)))
    vmax = float(scale * rng.uniform(0.05, 0.5))
    vmin = float(vmax * rng.uniform(0.0, 0.6))
    prm = dict(sep=sep, ali=ali, coh=coh, vmax=vmax, vmin=vmin)
    return n, field, prm, TUNINGS[int(rng.integers(len(TUNINGS)))]


def _check(sim, O, p, engine, pos, vel, what):
    sim.update(STEPS)
    if engine == "grid":
        op, ov = pos.copy(), vel.copy()
        of = O.GridPort(p, op).step(op, ov, STEPS, forces=True)
    else:
        op, ov = pos.copy(), vel.copy()
        of = O.step_allpairs(p, op, ov, STEPS, forces=True)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions, " + what)
    assert_bits_equal(gv, ov, "velocities, " + what)
    assert_bits_equal(sim.forces(), of, "forces, " + what)


@pytest.mark.parametrize("seed", range(100, 124))
def test_random_grid_configuration(boids_lib, oracle_mod, seed):
    O = oracle_mod
    n, field, prm, tuning = draw(seed)
    p = make_params(O, n, field, prm)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    sim.set_tuning(*tuning)
    sim.initialization_type = "random_uniform"
    sim.rand_seed = seed
    sim.init()
    pos, vel = O.init_state(p, "random_uniform", True, seed)
    what = "n=%d F=%.4g %r tuning %r" % (n, field, prm, tuning)
    _check(sim, O, p, "grid", pos, vel, what)
    # and from a gathered state: positions drawn around a few centres
    rng = np.random.default_rng(seed + 1)
    centres = rng.random((4, 3)) * field
    q = (centres[rng.integers(4, size=n)] + rng.normal(0, 0.04 * field, (n, 3))) % field
    q = q.astype(np.float32).reshape(-1)
    q[q >= np.float32(field)] = 0.0
    v = (vel.reshape(-1, 3) * rng.uniform(0.5, 1.5, (n, 1))).astype(np.float32).reshape(-1)
    sim.set_state(q, v)
    _check(sim, O, p, "grid", q, v, what + ", gathered")
    sim.close()


@pytest.mark.parametrize("seed", range(200, 208))
def test_random_allpairs_configuration(boids_lib, oracle_mod, seed):
    O = oracle_mod
    n, field, prm, tuning = draw(seed)
    n = min(n, 3000)  # the oracle tests every pair
    p = make_params(O, n, field, prm)
    for kernels in ("allpairs", "pairs"):
        sim = make_sim(boids_lib, kernels, n, field, prm)
        rng = np.random.default_rng(seed)
        pos = (rng.random((n, 3)) * field).astype(np.float32).reshape(-1)
        pos[pos >= np.float32(field)] = 0.0
        vel = (rng.normal(0, prm["vmax"], (n, 3))).astype(np.float32).reshape(-1)
        what = "%s n=%d F=%.4g %r" % (kernels, n, field, prm)
        sim.set_state(pos, vel)
        _check(sim, O, p, "allpairs", pos, vel, what)
        # some boids outside the field: the engine's own kernels take them
        q = pos.copy().reshape(-1, 3)
        k = max(1, n // 20)
        q[:k, int(rng.integers(3))] += np.float32(field * rng.uniform(0.01, 0.5))
        q[k:2 * k, int(rng.integers(3))] -= np.float32(field * rng.uniform(0.01, 0.5))
        q = q.reshape(-1)
        sim.set_state(q, vel)
        _check(sim, O, p, "allpairs", q, vel, what + ", partly outside")
        sim.close()
