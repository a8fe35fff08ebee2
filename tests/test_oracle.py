"""The oracle pinned to the reference (CPU only).

* against the committed golden vectors (tests/golden, made by running the
  reference engine built from its own sources: tests/golden/make_golden.py);
* against the reference engine itself where oracle/_ref exists;
* internal consistency: grid engine == all-pairs engine, bucketed neighbour
  sets == all-pairs neighbour sets, drand48 == the C library's.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, assert_bits_equal, make_params

GOLDEN_FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def test_golden_vectors_present():
    assert len(GOLDEN_FILES) >= 5


def test_drand48_matches_c_library(oracle_mod):
    libc = C.CDLL(None)
    libc.drand48.restype = C.c_double
    libc.srand48.argtypes = [C.c_long]
    for seed in (12345, 0, 1, -7, 2 ** 31 - 1):
        libc.srand48(seed)
        st = C.c_uint64()
        oracle_mod.lib().orc_srand48(C.byref(st), seed)
        fn = oracle_mod.lib().orc_drand48
        fn.restype = C.c_double
        fn.argtypes = [C.POINTER(C.c_uint64)]
        for _ in range(1000):
            assert fn(C.byref(st)) == libc.drand48()


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=[os.path.basename(p)[:-4] for p in GOLDEN_FILES])
def test_oracle_reproduces_golden(oracle_mod, path):
    O = oracle_mod
    g = np.load(path)
    prm = getattr(O, str(g["settings"]))
    n, field, steps, engine = int(g["n"]), float(g["field"]), int(g["steps"]), str(g["engine"])
    p = make_params(O, n, field, prm)
    pos, vel = O.init_state(p, str(g["init"]), seeded=(engine == "grid"), seed=int(g["seed"]))
    assert_bits_equal(pos, g["pos0"], "initial positions")
    assert_bits_equal(vel, g["vel0"], "initial velocities")
    if engine == "grid":
        f = O.GridPort(p, pos).step(pos, vel, steps, forces=True)
        assert np.array_equal(O.ref_cells(p, pos), g["grid_index"])
    else:
        f = O.step_allpairs(p, pos, vel, steps, forces=True)
    assert_bits_equal(pos, g["pos"], "positions after %d steps" % steps)
    assert_bits_equal(vel, g["vel"], "velocities after %d steps" % steps)
    assert_bits_equal(f, g["force"], "get_force of the last step")


def test_grid_port_equals_allpairs(oracle_mod):
    O = oracle_mod
    for n, field, sname, steps in ((3000, 0.57, "MARUN2019", 40), (800, 1.0, "TEST_INI", 25)):
        p = make_params(O, n, field, getattr(O, sname))
        pos, vel = O.init_state(p, "random_uniform", True, 99)
        p2, v2 = pos.copy(), vel.copy()
        fa = O.step_allpairs(p, pos, vel, steps, forces=True)
        fg = O.GridPort(p, p2).step(p2, v2, steps, forces=True)
        assert_bits_equal(pos, p2)
        assert_bits_equal(vel, v2)
        assert_bits_equal(fa, fg)


def test_bucketed_neighbour_sets_equal_all_pairs(oracle_mod):
    O = oracle_mod
    n, field = 4000, 0.63
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 5)
    O.GridPort(p, pos).step(pos, vel, 80)
    c1, h1 = O.neighbor_sets(p, pos, vel, bucketed=True)
    c0, h0 = O.neighbor_sets(p, pos, vel, bucketed=False)
    assert np.array_equal(c1, c0) and np.array_equal(h1, h0)
    assert c1.sum() > 0


def test_fp64_restatement_is_close_to_fp32(oracle_mod):
    O = oracle_mod
    n, field = 4000, 0.63
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 5)
    f32 = O.GridPort(p, pos.copy()).step(pos.copy(), vel.copy(), 1, forces=True).reshape(n, 9)
    f64 = O.forces_f64(p, pos, vel)
    for r in range(3):
        a, b = f32[:, 3 * r:3 * r + 3].astype(np.float64), f64[:, 3 * r:3 * r + 3]
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b) + 1e-30


def test_reference_geometry_and_rejections(oracle_mod):
    O = oracle_mod
    m = O.MARUN2019
    for field, G in ((1.0, 9), (1.6, 15), (4.0, 39)):
        R, g, GS = O.grid_geometry(make_params(O, 10, field, m))
        assert g == G and R == np.float32(0.05)
    assert O.grid_geometry(make_params(O, 10, 0.1, m)) is None      # GRID_NUM == 0
    assert O.grid_geometry(make_params(O, 10, 0.15, m)) is not None  # GRID_NUM == 1


ref = pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref")),
                         reason="reference engine not built here (no reference sources)")


@ref
@pytest.mark.parametrize("engine", ["grid", "allpairs"])
def test_oracle_matches_reference_engine_live(oracle_mod, engine):
    O = oracle_mod
    if not O.ref_available(engine):
        pytest.skip("oracle/_ref missing")
    for n, field, sname, init, steps in ((2048, 0.5, "MARUN2019", "random_uniform", 25),
                                         (500, 1.0, "TEST_INI", "test", 30)):
        p = make_params(O, n, field, getattr(O, sname))
        eng = O.RefEngine(engine, p, init, 4242)
        eng.init(fresh_drand48=True)
        pos, vel = O.init_state(p, init, seeded=(engine == "grid"), seed=4242)
        rp, rv = eng.state()
        assert_bits_equal(pos, rp, "init")
        assert_bits_equal(vel, rv, "init")
        eng.update(steps)
        if engine == "grid":
            f = O.GridPort(p, pos).step(pos, vel, steps, forces=True)
            assert np.array_equal(O.ref_cells(p, pos), eng.grid_index())
        else:
            f = O.step_allpairs(p, pos, vel, steps, forces=True)
        rp, rv = eng.state()
        assert_bits_equal(pos, rp, "positions")
        assert_bits_equal(vel, rv, "velocities")
        assert_bits_equal(f, eng.forces(), "forces")
        eng.close()


def _edge_states(O):
    """(name, n, field, settings, pos, vel, steps) for degenerate inputs."""
    m = O.MARUN2019
    allround = dict(m, sep=(0.01, 1.0, 0.002), ali=(0.05, 1.5, 0.06), coh=(0.05, 2.0, 0.008))
    cases = []
    for n in (1, 2, 3):
        # a short file of boids heading along +x, each within the sight of
        # the ones behind it (the first two closer than the separation radius)
        pos = np.array([[0.40 + 0.008 * i + 0.01 * (i > 1), 0.50 + 0.002 * i, 0.30] for i in range(n)], np.float32)
        vel = np.array([[0.003, 0.0005 * i, 0.0002] for i in range(n)], np.float32)
        cases.append(("n=%d" % n, n, 1.0, m, pos.reshape(-1), vel.reshape(-1), 20))
    p = make_params(O, 512, 0.5, allround)
    pos, vel = O.init_state(p, "random_uniform", True, 5)
    cases.append(("all-round sight", 512, 0.5, allround, pos, vel, 20))
    # boids on the field's faces: coordinates exactly 0 and exactly F
    p = make_params(O, 256, 0.5, m)
    pos, vel = O.init_state(p, "random_uniform", True, 6)
    pos = pos.reshape(-1, 3)
    pos[0:16, 0] = 0.0
    pos[16:32, 1] = np.float32(0.5)
    pos[32:48] = np.float32(0.5)
    pos[48:64, 2] = 0.0
    cases.append(("faces", 256, 0.5, m, pos.reshape(-1), vel, 10))
    # coincident boids, zero velocities (the view cone's NaN) and speeds
    # outside [vmin, vmax] (both clamp branches)
    p = make_params(O, 192, 0.5, m)
    pos, vel = O.init_state(p, "random_uniform", True, 7)
    pos, vel = pos.reshape(-1, 3), vel.reshape(-1, 3)
    pos[1::8] = pos[0::8]
    vel[2::8] = 0.0
    vel[3::8] *= np.float32(4.0)
    vel[4::8] *= np.float32(0.25)
    cases.append(("coincident, still, fast and slow", 192, 0.5, m, pos.reshape(-1), vel.reshape(-1), 10))
    return cases


@ref
@pytest.mark.parametrize("engine", ["grid", "allpairs"])
def test_oracle_matches_reference_engine_on_edge_cases(oracle_mod, engine):
    """The oracle against the reference's own engine on degenerate inputs:
    one to three boids, all-round sight (angles >= 1), boids on the faces of
    the field (x == 0, x == F), coincident boids, boids at rest and speeds
    outside the limits."""
    O = oracle_mod
    if not O.ref_available(engine):
        pytest.skip("oracle/_ref missing")
    for name, n, field, prm, pos, vel, steps in _edge_states(O):
        p = make_params(O, n, field, prm)
        eng = O.RefEngine(engine, p, "random_uniform", 1)
        eng.set_state(pos, vel)
        pos, vel = pos.copy(), vel.copy()
        eng.update(steps)
        if engine == "grid":
            f = O.GridPort(p, pos).step(pos, vel, steps, forces=True)
            assert np.array_equal(O.ref_cells(p, pos), eng.grid_index()), name
        else:
            f = O.step_allpairs(p, pos, vel, steps, forces=True)
        rp, rv = eng.state()
        assert_bits_equal(pos, rp, name + ": positions")
        assert_bits_equal(vel, rv, name + ": velocities")
        assert_bits_equal(f, eng.forces(), name + ": forces")
        eng.close()
