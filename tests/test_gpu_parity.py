"""GPU parity: the CUDA engines against the oracle, through the C ABI.

The bar is bit-for-bit equality with the reference's FP32 arithmetic (the
oracle restates it and is itself pinned bit-for-bit to the reference engine
compiled from its sources, see test_oracle.py).  Trajectories are compared
bit-for-bit over the step counts of the reference's own test scripts
(test/compare_grid.sh: N=100 T=30, test/compare_legacy.sh: N=1000 T=30).
"""
import numpy as np
import pytest

from conftest import assert_bits_equal, make_params, make_sim

pytestmark = pytest.mark.gpu

CASES = [
    # name, n, field, settings, init, steps
    ("compare_grid_sh", 100, 1.0, "TEST_INI", "test", 30),
    ("compare_legacy_sh", 1000, 1.0, "TEST_INI", "test", 30),
    ("marun2019_F0.5", 2048, 0.5, "MARUN2019", "random_uniform", 50),
    ("marun2019_config0", 16384, 1.0, "MARUN2019", "random_uniform", 10),
]


def _oracle_run(O, p, engine, pos, vel, steps):
    pos, vel = pos.copy(), vel.copy()
    if engine == "grid":
        f = O.GridPort(p, pos).step(pos, vel, steps, forces=True)
    else:
        f = O.step_allpairs(p, pos, vel, steps, forces=True)
    return pos, vel, f


@pytest.mark.parametrize("engine", ["grid", "allpairs", "pairs"])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_trajectory_bit_exact(boids_lib, oracle_mod, engine, case):
    name, n, field, sname, init, steps = case
    O = oracle_mod
    prm = getattr(O, sname)
    if engine != "grid" and n > 4096:  # the oracle tests every pair
        steps = 3
    p = make_params(O, n, field, prm)
    sim = make_sim(boids_lib, engine, n, field, prm)
    sim.initialization_type = init
    sim.init()  # the engine's own seeding rule, as in the reference
    pos0, vel0 = O.init_state(p, init, seeded=(engine == "grid"), seed=12345)
    gp, gv = sim.state()
    assert_bits_equal(gp, pos0, "init positions")
    assert_bits_equal(gv, vel0, "init velocities")
    sim.update(steps)
    gp, gv = sim.state()
    gf = sim.forces()
    op, ov, of = _oracle_run(O, p, engine, pos0, vel0, steps)
    assert_bits_equal(gp, op, "positions after %d steps" % steps)
    assert_bits_equal(gv, ov, "velocities after %d steps" % steps)
    assert_bits_equal(gf, of, "forces of step %d" % steps)


@pytest.mark.parametrize("engine", ["grid", "allpairs", "pairs"])
def test_single_step_forces_from_identical_state(boids_lib, oracle_mod, engine):
    """The same evolved state is fed to both sides; one step's get_force must match."""
    O = oracle_mod
    n, field = 16384, 1.0
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 7)
    O.GridPort(p, pos).step(pos, vel, 120)  # clustered, realistic state
    sim = make_sim(boids_lib, engine, n, field, O.MARUN2019)
    sim.set_state(pos, vel)
    sim.update(1)
    op, ov, of = _oracle_run(O, p, "grid", pos, vel, 1)
    assert_bits_equal(sim.forces(), of, "forces")
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")


def test_grid_equals_allpairs_on_gpu(boids_lib, oracle_mod):
    O = oracle_mod
    n, field = 8192, 0.8
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos, vel = O.init_state(p, "random_uniform", True, 99)
    a = make_sim(boids_lib, "grid", n, field, prm)
    b = make_sim(boids_lib, "allpairs", n, field, prm)
    a.set_state(pos, vel)
    b.set_state(pos, vel)
    a.update(20)
    b.update(20)
    ap, av = a.state()
    bp, bv = b.state()
    assert_bits_equal(ap, bp, "positions")
    assert_bits_equal(av, bv, "velocities")


def test_reference_cells_bit_exact(boids_lib, oracle_mod):
    """Boid::grid_index (primary + overlapped cells) equals the reference's."""
    O = oracle_mod
    n, field = 65536, 1.6
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 12345)
    sim = make_sim(boids_lib, "grid", n, field, O.MARUN2019)
    sim.set_state(pos, vel)
    sim.update(5)
    gp, gv = sim.state()
    cells = sim.cells()
    ref = O.ref_cells(p, gp.reshape(-1))
    assert np.array_equal(cells, ref)
    info = sim.grid_info()
    assert info["ref_grid_num"] == 15
    assert O.grid_geometry(p)[1] == 15


@pytest.mark.parametrize("engine", ["grid", "allpairs", "pairs"])
def test_neighbor_sets_bit_exact(boids_lib, oracle_mod, engine):
    O = oracle_mod
    n, field = 32768, 1.27
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 3)
    O.GridPort(p, pos).step(pos, vel, 60)
    sim = make_sim(boids_lib, engine, n, field, O.MARUN2019)
    sim.set_state(pos, vel)
    c, h = sim.neighbor_sets()
    oc, oh = O.neighbor_sets(p, pos, vel)
    assert np.array_equal(c, oc)
    assert np.array_equal(h, oh)
    # the diagnostic does not advance or disturb the state
    gp, gv = sim.state()
    assert_bits_equal(gp, pos, "state after diagnostics")
    sim.update(1)
    op, ov, of = _oracle_run(O, p, "grid", pos, vel, 1)
    assert_bits_equal(sim.state()[0], op, "step after diagnostics")


@pytest.mark.parametrize("engine", ["grid", "allpairs", "pairs"])
def test_dense_cluster_overflow_paths(boids_lib, oracle_mod, engine):
    """Hundreds of neighbours per boid: more than the per-thread list holds
    (grid: several sorted passes; all-pairs: ordered full scan)."""
    O = oracle_mod
    rng = np.random.default_rng(5)
    n, field = 600, 1.0
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos = (0.5 + 0.02 * rng.standard_normal((n, 3))).astype(np.float32).reshape(-1)
    pos[: 3 * 50] = rng.random(3 * 50, dtype=np.float32)  # some isolated boids
    vel = (0.003 * rng.standard_normal((n, 3))).astype(np.float32).reshape(-1)
    sim = make_sim(boids_lib, engine, n, field, prm)
    sim.set_state(pos, vel)
    sim.update(3)
    op, ov, of = _oracle_run(O, p, "allpairs", pos, vel, 3)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


def test_huge_cells_in_id_windows(boids_lib, oracle_mod):
    """Neighbourhoods of thousands of boids (more than the dense kernel's
    shared list): the cell is done in ascending id windows, its boids' sums
    carried from window to window, over several rounds of 128 boids."""
    O = oracle_mod
    rng = np.random.default_rng(23)
    n, field = 20000, 1.0
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos = rng.random((n, 3), dtype=np.float32)
    ball = rng.permutation(n)[:9000]  # ids spread over the whole range
    pos[ball] = (0.5 + 0.012 * rng.standard_normal((ball.size, 3))).astype(np.float32)
    pos[ball[:3000]] = (0.18 + 0.02 * rng.standard_normal((3000, 3))).astype(np.float32)
    pos = pos.reshape(-1)
    vel = (0.003 * rng.standard_normal((n, 3))).astype(np.float32).reshape(-1)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    sim.set_state(pos, vel)
    sim.update(2)
    op, ov, of = _oracle_run(O, p, "grid", pos, vel, 2)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


@pytest.mark.slow
def test_huge_cell_window_narrowing(boids_lib, oracle_mod):
    """More ids in the flock than the window search's bins times the shared
    list's capacity (2048 x 1024), so one histogram bin spans more ids than
    the list holds; a ball of consecutive ids makes the first bin overflow
    and the search narrow to it."""
    O = oracle_mod
    rng = np.random.default_rng(29)
    n = 8_500_000
    field = float(np.float32((n / 16384.0) ** (1.0 / 3.0)))
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos = (rng.random((n, 3), dtype=np.float32) * np.float32(field)).astype(np.float32)
    pos[:2600] = (np.float32(field / 2) + 0.01 * rng.standard_normal((2600, 3))).astype(np.float32)
    pos = pos.reshape(-1)
    vel = (0.003 * rng.standard_normal((n, 3))).astype(np.float32).reshape(-1)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    sim.set_state(pos, vel)
    sim.update(1)
    op, ov, of = _oracle_run(O, p, "grid", pos, vel, 1)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


@pytest.mark.parametrize("engine", ["grid", "allpairs", "pairs"])
def test_degenerate_pairs(boids_lib, oracle_mod, engine):
    """Coincident boids (distance 0), zero velocities (0/0 in the cone test),
    boids on the periodic faces and at x == field_size exactly."""
    O = oracle_mod
    n, field = 64, 1.0
    prm = dict(O.MARUN2019)
    p = make_params(O, n, field, prm)
    rng = np.random.default_rng(11)
    pos = rng.random((n, 3), dtype=np.float32)
    vel = (0.004 * rng.standard_normal((n, 3))).astype(np.float32)
    pos[1] = pos[0]                      # coincident
    vel[2] = 0.0                         # no heading
    pos[3] = [0.0, 0.5, 0.5]; pos[4] = [np.float32(field), 0.5, 0.5]  # across x faces
    pos[5] = [0.999, 0.001, 0.0]; pos[6] = [0.001, 0.999, 0.9995]
    pos[7] = [0.5, 0.0, np.float32(field)]
    vel[3] = [-0.004, 0, 0]
    sim = make_sim(boids_lib, engine, n, field, prm)
    sim.set_state(pos, vel)
    sim.update(4)
    op, ov, of = _oracle_run(O, p, "allpairs", pos.reshape(-1), vel.reshape(-1), 4)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


def _perpendicular_groups(n_groups, field, seed):
    """Groups of 8 boids: a centre and 7 neighbours placed at right angles
    to the centre's velocity, give or take a few ulps, so that the exact
    v . r of many pairs is 0 or within rounding of it; a quarter of the
    groups straddle a periodic face."""
    rng = np.random.default_rng(seed)
    pos, vel = [], []
    for g in range(n_groups):
        c = rng.random(3) * field
        if g % 4 == 0:
            c[g // 4 % 3] = field * rng.choice([0.0, 0.9995, 0.0004])
        v = rng.standard_normal(3)
        v *= rng.uniform(0.001, 0.005) / np.linalg.norm(v)
        vh = v / np.linalg.norm(v)
        pos.append(c)
        vel.append(v)
        for k in range(7):
            u = np.cross(vh, rng.standard_normal(3))
            u /= np.linalg.norm(u)
            eps = rng.choice([0.0, 1e-9, -1e-9, 3e-8, -3e-8, 1e-7, -1e-7])
            pos.append(np.mod(c + rng.uniform(0.003, 0.0499) * u + eps * vh, field))
            vel.append(rng.standard_normal(3) * 0.003)
    pos = np.asarray(pos, np.float32)
    pos[pos >= np.float32(field)] = 0.0
    return pos, np.asarray(vel, np.float32)


@pytest.mark.parametrize("tuning", [None, (1 << 30, 1 << 30, 1 << 30, 1 << 30), (1, 1, 0, 0)],
                         ids=["default", "all_sparse", "all_dense"])
def test_view_cone_pretest_at_right_angles(boids_lib, oracle_mod, tuning):
    """The candidate filters drop pairs behind a boid (approximate v . r
    below -|v| * dot_eps) before the exact tests; pairs at right angles to
    the velocity, within rounding of v . r = 0, are the ones that pre-test
    could get wrong.  Neighbour sets, forces and the next state must equal
    the oracle's."""
    O = oracle_mod
    field = 1.0
    pos, vel = _perpendicular_groups(512, field, 23)
    n = pos.shape[0]
    prm = dict(O.MARUN2019)
    p = make_params(O, n, field, prm)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    if tuning:
        sim.set_tuning(*tuning)
    sim.set_state(pos, vel)
    cnt, hsh = sim.neighbor_sets()
    ocnt, ohsh = O.neighbor_sets(p, pos.reshape(-1), vel.reshape(-1))
    assert np.array_equal(cnt, ocnt) and np.array_equal(hsh, ohsh)
    sim.update(2)
    op, ov, of = _oracle_run(O, p, "allpairs", pos.reshape(-1), vel.reshape(-1), 2)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


@pytest.mark.parametrize("tuning", [None, (1, 1, 0, 0)], ids=["default", "all_dense"])
def test_cells_much_larger_than_the_radius(boids_lib, oracle_mod, tuning):
    """A large field caps the grid at 128 cells per axis, so cells are three
    times the radius: the half-precision filter's margins are then relatively
    wider.  A gathered cluster with a quarter of the boids well over vmax
    (the filter's view-cone pre-test is off for those) and the rest at rest
    or in motion; one and three updates against the oracle."""
    O = oracle_mod
    n, field = 4096, 20.0
    prm = dict(O.MARUN2019)
    p = make_params(O, n, field, prm)
    rng = np.random.default_rng(31)
    pos = (rng.random((n, 3)) * 0.3 + 9.85).astype(np.float32)
    pos[: n // 8] = (rng.random((n // 8, 3)) * field).astype(np.float32)
    vel = (0.003 * rng.standard_normal((n, 3))).astype(np.float32)
    vel[n // 4: n // 2] *= 20.0
    vel[-16:] = 0.0
    sim = make_sim(boids_lib, "grid", n, field, prm)
    assert sim.grid_info()["dev_cells_per_axis"] == 128
    if tuning:
        sim.set_tuning(*tuning)
    sim.set_state(pos, vel)
    cnt, hsh = sim.neighbor_sets()
    ocnt, ohsh = O.neighbor_sets(p, pos.reshape(-1), vel.reshape(-1))
    assert np.array_equal(cnt, ocnt) and np.array_equal(hsh, ohsh)
    assert cnt[:, 0].mean() > 20
    sim.update(3)
    op, ov, of = _oracle_run(O, p, "allpairs", pos.reshape(-1), vel.reshape(-1), 3)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


def test_allpairs_engine_kernel_choice(boids_lib, oracle_mod):
    """The all-pairs engine runs the grid kernels for states inside the field
    and its own N^2 kernels for states outside it (the reference takes
    those: its minimum image then decides); both match the oracle's
    all-pairs update bit for bit."""
    O = oracle_mod
    n, field = 2000, 1.0
    prm = dict(O.MARUN2019)
    p = make_params(O, n, field, prm)
    rng = np.random.default_rng(41)
    pos = rng.random((n, 3), dtype=np.float32)
    vel = (0.004 * rng.standard_normal((n, 3))).astype(np.float32)
    sim = make_sim(boids_lib, "allpairs", n, field, prm)
    for outside in (False, True, False):
        q = pos.copy()
        if outside:
            q[:40, 0] += np.float32(field)      # beyond the far face
            q[40:80, 1] -= np.float32(0.25)     # below zero
        sim.set_state(q, vel)
        assert sim.grid_info()["list_capacity"] == (256 if outside else 12)
        sim.update(3)
        op, ov, of = _oracle_run(O, p, "allpairs", q.reshape(-1), vel.reshape(-1), 3)
        gp, gv = sim.state()
        assert_bits_equal(gp, op, "positions (outside=%s)" % outside)
        assert_bits_equal(gv, ov, "velocities (outside=%s)" % outside)
        assert_bits_equal(sim.forces(), of, "forces (outside=%s)" % outside)


def test_grid_engine_refuses_states_outside_the_field(boids_lib, oracle_mod):
    """The grid engine bins positions in [0, F]: boids_set_state refuses a
    state with a coordinate outside it, or NaN, wherever that boid sits among
    the pieces the state is copied in, and the handle is then without a
    state.  Coordinates 0 and F are inside.  A good state set afterwards
    runs bit-exact."""
    O = oracle_mod
    n, field = 5000, 1.0
    p = make_params(O, n, field, O.MARUN2019)
    rng = np.random.default_rng(7)
    pos = rng.random((n, 3), dtype=np.float32)
    vel = (0.004 * rng.standard_normal((n, 3))).astype(np.float32)
    sim = make_sim(boids_lib, "grid", n, field, O.MARUN2019)
    sim.set_state(pos, vel)
    sim.update(1)
    above = np.nextafter(np.float32(field), np.float32(2))
    for i, c, v in ((0, 0, np.float32(-1e-7)), (2047, 1, above), (3100, 0, np.float32(np.inf)),
                    (4999, 2, np.float32(np.nan))):
        q = pos.copy()
        q[i, c] = v
        with pytest.raises(boids_lib.BoidsError, match="positions must lie"):
            sim.set_state(q, vel)
        with pytest.raises(boids_lib.BoidsError, match="no state"):
            sim.update(1)
    q = pos.copy()
    q[10] = field
    q[4998] = 0.0
    sim.set_state(q, vel)
    assert_bits_equal(sim.state()[0], q, "positions on the faces")
    sim.set_state(pos, vel)
    sim.update(3)
    op, ov, of = _oracle_run(O, p, "grid", pos.reshape(-1), vel.reshape(-1), 3)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")
    sim.close()


def test_all_round_angles_and_test_ini(boids_lib, oracle_mod):
    """Sight angles >= 1 skip the cone test entirely (src/boid.cpp:29-31)."""
    O = oracle_mod
    prm = dict(sep=(0.02, 1.0, 0.001), ali=(0.05, 1.5, 0.05), coh=(0.05, 0.2, 0.01),
               vmax=0.004, vmin=0.0005)
    n, field = 4096, 0.6
    p = make_params(O, n, field, prm)
    pos, vel = O.init_state(p, "random_uniform", True, 1)
    for engine in ("grid", "allpairs", "pairs"):
        sim = make_sim(boids_lib, engine, n, field, prm)
        sim.set_state(pos, vel)
        sim.update(10)
        op, ov, of = _oracle_run(O, p, "allpairs", pos, vel, 10)
        assert_bits_equal(sim.state()[0], op, engine)
        assert_bits_equal(sim.forces(), of, engine)


@pytest.mark.parametrize("n", [0, 1, 2, 33])
def test_tiny_populations(boids_lib, oracle_mod, n):
    O = oracle_mod
    for engine in ("grid", "allpairs", "pairs"):
        p = make_params(O, n, 1.0, O.MARUN2019)
        sim = make_sim(boids_lib, engine, n, 1.0, O.MARUN2019)
        sim.init()
        pos, vel = O.init_state(p, "random_uniform", engine == "grid", 12345)
        sim.update(5)
        op, ov, of = _oracle_run(O, p, "allpairs", pos, vel, 5)
        gp, gv = sim.state()
        assert_bits_equal(gp, op, "positions")
        assert_bits_equal(gv, ov, "velocities")


def test_fp64_oracle_tolerance(boids_lib, oracle_mod):
    """Per-rule force error of the FP32 step against the FP64 restatement.

    Tolerance, written here: for each rule the aggregate (Frobenius) relative
    error over all boids is <= 1e-5, and every boid's error is <= 1e-4 of the
    rule's operand scale (cohesion: c*max(|x_i|, |mean x_j|); separation:
    c*n_sep; alignment: c*max(|v_i|, |mean v_j|)).  The per-boid plain
    relative error can exceed 1e-5 for cohesion: the reference forms
    mean(x_j) - x_i in float, which cancels; the GPU is bit-identical to the
    reference, so it inherits exactly that error.
    """
    O = oracle_mod
    n, field = 65536, 1.6
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos, vel = O.init_state(p, "random_uniform", True, 12345)
    O.GridPort(p, pos).step(pos, vel, 50)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    sim.set_state(pos, vel)
    sim.update(1)
    f32 = sim.forces().astype(np.float64)
    f64 = O.forces_f64(p, pos, vel)
    cnt, _ = O.neighbor_sets(p, pos, vel)
    P = pos.reshape(n, 3).astype(np.float64)
    V = vel.reshape(n, 3).astype(np.float64)
    cc, cs, ca = prm["coh"][2], prm["sep"][2], prm["ali"][2]
    scale = [cc * np.maximum(np.linalg.norm(P, axis=1), np.linalg.norm(f64[:, 0:3] / cc + P, axis=1)),
             cs * cnt[:, 1],
             ca * np.maximum(np.linalg.norm(V, axis=1), np.linalg.norm(f64[:, 6:9] / ca + V, axis=1))]
    for r in range(3):
        a, b = f32[:, 3 * r:3 * r + 3], f64[:, 3 * r:3 * r + 3]
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b) + 1e-30
        err = np.linalg.norm(a - b, axis=1)
        s = scale[r]
        assert np.all(err[s == 0] == 0)
        assert np.all(err[s > 0] <= 1e-4 * s[s > 0])


def _polarization(vel):
    v = np.asarray(vel, np.float64).reshape(-1, 3)
    sp = np.linalg.norm(v, axis=1)
    return float(np.linalg.norm((v / np.where(sp > 0, sp, 1)[:, None]).sum(0)) / v.shape[0])


@pytest.mark.slow
def test_allpairs_65536_trajectory_and_polarization(boids_lib, oracle_mod):
    """The all-pairs workload at N=65536, F=1.6 from the reference's
    (unseeded) all-pairs init: 1000 updates on the grid kernels and on the
    N^2 kernels give the same bits at every 50th step (so the same
    polarization history), and the first 200 updates equal the oracle's bit
    for bit (its grid port, itself equal to its all-pairs update)."""
    O = oracle_mod
    n, field = 65536, 1.6
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    sims = [make_sim(boids_lib, e, n, field, prm, record_forces=False) for e in ("allpairs", "pairs")]
    for s in sims:
        s.init()
    pos, vel = O.init_state(p, "random_uniform", False, 12345)
    assert_bits_equal(sims[0].state()[0], pos, "init")
    port = O.GridPort(p, pos)
    pol = []
    for t in range(50, 1001, 50):
        for s in sims:
            s.update(50)
        (pa, va), (pb, vb) = sims[0].state(), sims[1].state()
        assert_bits_equal(pa, pb, "grid vs N^2 kernels, step %d" % t)
        assert_bits_equal(va, vb, "grid vs N^2 kernels, step %d" % t)
        if t <= 200:
            port.step(pos, vel, 50)
            assert_bits_equal(pa, pos, "oracle positions, step %d" % t)
            assert_bits_equal(va, vel, "oracle velocities, step %d" % t)
        pol.append(_polarization(va))
    assert pol[-1] > pol[0] > 0.0  # the flock aligns as it gathers


# ---------------------------------------------------------------- golden vectors of the reference

import glob as _glob
import os as _os

from conftest import GOLDEN as _GOLDEN

_GOLDEN_FILES = sorted(_glob.glob(_os.path.join(_GOLDEN, "*.npz")))


@pytest.mark.parametrize("path", _GOLDEN_FILES, ids=[_os.path.basename(p)[:-4] for p in _GOLDEN_FILES])
def test_gpu_reproduces_reference_golden(boids_lib, oracle_mod, path):
    """The reference engine's own outputs (tests/golden/make_golden.py), from its initial state."""
    O = oracle_mod
    g = np.load(path)
    prm = getattr(O, str(g["settings"]))
    n, field, steps, engine = int(g["n"]), float(g["field"]), int(g["steps"]), str(g["engine"])
    sim = make_sim(boids_lib, engine, n, field, prm)
    sim.set_state(g["pos0"], g["vel0"])
    sim.update(steps)
    gp, gv = sim.state()
    assert_bits_equal(gp, g["pos"], "positions")
    assert_bits_equal(gv, g["vel"], "velocities")
    assert_bits_equal(sim.forces(), g["force"], "get_force")
    if engine == "grid":
        assert np.array_equal(sim.cells(), g["grid_index"])


@pytest.mark.parametrize("path", _GOLDEN_FILES, ids=[_os.path.basename(p)[:-4] for p in _GOLDEN_FILES])
def test_host_init_reproduces_reference_golden(boids_lib, oracle_mod, path):
    """BoidSimulation::init's drand48 draws (host side of the library)."""
    O = oracle_mod
    g = np.load(path)
    prm = getattr(O, str(g["settings"]))
    sim = make_sim(boids_lib, str(g["engine"]), int(g["n"]), float(g["field"]), prm)
    sim.initialization_type = str(g["init"])
    sim.rand_seed = int(g["seed"])
    sim.init()
    gp, gv = sim.state()
    assert_bits_equal(gp, g["pos0"], "initial positions")
    assert_bits_equal(gv, g["vel0"], "initial velocities")


@pytest.mark.parametrize("tuning", [(1, 1, 0, 0), (1 << 30, 1 << 30, 1 << 30, 1 << 30), (4, 2, 64, 128)])
def test_dense_thresholds_do_not_change_results(boids_lib, oracle_mod, tuning):
    """Every cell to the CTA-per-cell kernel, every boid to the per-boid
    kernel (cells over the shared list still go dense, in id windows), and a
    mix: the same bits as the oracle."""
    O = oracle_mod
    rng = np.random.default_rng(41)
    n, field = 6000, 0.9
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos = rng.random((n, 3), dtype=np.float32) * np.float32(field)
    pos[:2500] = (0.45 + 0.03 * rng.standard_normal((2500, 3))).astype(np.float32)
    pos = pos.reshape(-1)
    vel = (0.003 * rng.standard_normal((n, 3))).astype(np.float32).reshape(-1)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    sim.set_tuning(*tuning)
    assert sim.tuning() == tuple(tuning)
    sim.set_state(pos, vel)
    sim.update(3)
    op, ov, of = _oracle_run(O, p, "grid", pos, vel, 3)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")


def test_handle_autotune_keeps_the_trajectory(boids_lib, oracle_mod):
    O = oracle_mod
    prm = O.MARUN2019
    n, field = 20000, 1.08
    a = make_sim(boids_lib, "grid", n, field, prm)
    b = make_sim(boids_lib, "grid", n, field, prm)
    for s in (a, b):
        s.init()
        s.update(40)
    t = a.autotune(2)
    assert len(t) == 4
    pa, va = a.state()
    pb, vb = b.state()
    assert_bits_equal(pa, pb, "state after autotune")
    a.update(25)
    b.update(25)
    pa, va = a.state()
    pb, vb = b.state()
    assert_bits_equal(pa, pb, "positions")
    assert_bits_equal(va, vb, "velocities")


@pytest.mark.parametrize("engine", ["grid", "allpairs", "pairs"])
def test_graph_replayed_steps_equal_single_steps(boids_lib, oracle_mod, engine):
    """boids_step(sim, k >= 32) replays captured 16-update graphs, and the
    grid engine's other updates replay a one-update graph; the same updates
    launched directly, one call at a time (phase timing on, which launches
    every kernel itself), give the same bits and the same launch count."""
    O = oracle_mod
    prm = O.MARUN2019
    n, field = (12000, 0.91) if engine == "grid" else (3000, 0.6)
    a = make_sim(boids_lib, engine, n, field, prm)
    b = make_sim(boids_lib, engine, n, field, prm)
    for s in (a, b):
        s.init()
    b.profile_enable(True)
    la, lb = a.kernel_launches(), b.kernel_launches()
    a.update(70)          # 4 replays of 16 updates + 6 single updates
    for _ in range(70):
        b.update(1)
    pa, va = a.state()
    pb, vb = b.state()
    assert_bits_equal(pa, pb, "positions")
    assert_bits_equal(va, vb, "velocities")
    assert_bits_equal(a.forces(), b.forces(), "forces")
    assert a.kernel_launches() - la == b.kernel_launches() - lb
    a.set_tuning(4, 2, 64, 128)  # new constants: the graph is captured again
    b.set_tuning(4, 2, 64, 128)
    a.update(40)
    for _ in range(40):
        b.update(1)
    assert_bits_equal(a.state()[0], b.state()[0], "positions after retuning")
    for _ in range(5):   # single updates
        a.update(1)
    b.update(5)
    assert_bits_equal(a.state()[0], b.state()[0], "positions after single updates")
    assert_bits_equal(a.forces(), b.forces(), "forces after single updates")


@pytest.mark.parametrize("engine", ["grid", "allpairs"])
def test_c_caller_frames_equal_the_oracle(capi_caller, oracle_mod, tmp_path, engine):
    """tests/native/capi_caller.c drives the library from C the way the
    reference's frame loop drives BoidSimulation (src/main.cpp:187-291): the
    frame of each step's state, double-buffered while the update runs, then
    the final state and get_force values.  Every frame equals the oracle."""
    import subprocess
    O = oracle_mod
    n, field, steps = 2048, 0.5, 20
    out = tmp_path / "frames.bin"
    r = subprocess.run([capi_caller, str(n), str(field), str(steps), str(out), engine],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data = np.fromfile(out, dtype=np.float32)
    assert data.size == (steps + 5) * 3 * n
    frames = data[:steps * 3 * n].reshape(steps, n, 3)
    tail = data[steps * 3 * n:]
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 12345)
    grid = O.GridPort(p, pos) if engine == "grid" else None
    for t in range(steps):
        assert_bits_equal(frames[t], pos, "frame %d" % t)
        f = grid.step(pos, vel, 1, forces=True) if grid else O.step_allpairs(p, pos, vel, 1, forces=True)
    assert_bits_equal(tail[:3 * n], pos, "final positions")
    assert_bits_equal(tail[3 * n:6 * n], vel, "final velocities")
    assert_bits_equal(tail[6 * n:], f, "forces of the last update")


def test_crowded_cell_with_bunched_ids(boids_lib, oracle_mod):
    """A crowded cell whose boids' ids bunch at both ends of the id range
    (0..149 and N-150..N-1): the CTA-per-cell kernel's id sort sees a few
    buckets holding most of its candidates and takes its radix path; the
    cells elsewhere take the bucket path.  Three updates against the oracle."""
    O = oracle_mod
    rng = np.random.default_rng(7)
    n, field = 65536, 1.6
    prm = O.MARUN2019
    p = make_params(O, n, field, prm)
    pos = rng.random((n, 3)) * field
    crowd = np.r_[np.arange(150), np.arange(n - 150, n)]
    d = rng.normal(size=(crowd.size, 3))
    d *= (0.02 * rng.uniform(0, 1, (crowd.size, 1)) ** (1 / 3)) / np.linalg.norm(d, axis=1, keepdims=True)
    pos[crowd] = 0.8 + d
    pos = pos.astype(np.float32).reshape(-1)
    v = rng.normal(size=(n, 3))
    vel = (v * rng.uniform(0.001, 0.005, (n, 1)) / np.linalg.norm(v, axis=1, keepdims=True))
    vel = vel.astype(np.float32).reshape(-1)
    sim = make_sim(boids_lib, "grid", n, field, prm)
    sim.set_state(pos, vel)
    sim.update(3)
    op, ov, of = _oracle_run(O, p, "grid", pos, vel, 3)
    gp, gv = sim.state()
    assert_bits_equal(gp, op, "positions")
    assert_bits_equal(gv, ov, "velocities")
    assert_bits_equal(sim.forces(), of, "forces")
