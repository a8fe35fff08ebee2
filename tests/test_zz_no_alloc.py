"""boids_step_noalloc, the update for callers that cannot let the library
allocate device memory (their GPU memory is owned by their own pool or budget,
or their loop must not meet cudaMalloc/cudaFree).  It must give the same
result as the handle API, call after call, although every call reuses one
shared static scratch array.

This file runs last on purpose (pytest collects files alphabetically), so a
failure here still leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_bits_equal, make_params, make_sim

pytestmark = pytest.mark.gpu


def _params(B, n, field, prm):
    return B.Params(n, field, *prm["sep"], *prm["ali"], *prm["coh"], prm["vmax"], prm["vmin"],
                    B.ENGINE_GRID, 0, 0, 0)


def test_noalloc_step_matches_handle_api_twice(boids_lib, oracle_mod):
    torch = pytest.importorskip("torch")
    B, O = boids_lib, oracle_mod
    n, field = 4096, 0.63
    prm = O.MARUN2019
    pos0, vel0 = O.init_state(make_params(O, n, field, prm), "random_uniform", True, 12345)

    # the existing entry points: a handle, two updates
    sim = make_sim(B, "grid", n, field, prm, record_forces=False)
    sim.set_state(pos0, vel0)
    sim.update(1)
    p1, v1 = sim.state()
    sim.update(1)
    p2, v2 = sim.state()
    sim.close()

    # the allocation-free entry point, two calls in a row on caller-owned device arrays
    dev = torch.device("cuda", 0)
    a_pos = torch.from_numpy(pos0.copy()).to(dev)
    a_vel = torch.from_numpy(vel0.copy()).to(dev)
    b_pos = torch.empty_like(a_pos)
    b_vel = torch.empty_like(a_vel)
    prms = _params(B, n, field, prm)
    L = B.lib()
    torch.cuda.synchronize()
    rc = L.boids_step_noalloc(C.byref(prms), a_pos.data_ptr(), a_vel.data_ptr(),
                              b_pos.data_ptr(), b_vel.data_ptr(), None)
    assert rc == 0, L.boids_last_error().decode()
    torch.cuda.synchronize()
    assert_bits_equal(b_pos.cpu().numpy(), p1, "positions, call 1")
    assert_bits_equal(b_vel.cpu().numpy(), v1, "velocities, call 1")
    rc = L.boids_step_noalloc(C.byref(prms), b_pos.data_ptr(), b_vel.data_ptr(),
                              a_pos.data_ptr(), a_vel.data_ptr(), None)
    assert rc == 0, L.boids_last_error().decode()
    torch.cuda.synchronize()
    assert_bits_equal(a_pos.cpu().numpy(), p2, "positions, call 2")
    assert_bits_equal(a_vel.cpu().numpy(), v2, "velocities, call 2")


def test_noalloc_refuses_sizes_beyond_its_scratch(boids_lib):
    B = boids_lib
    from oracle import MARUN2019 as prm
    n = 1 << 20
    prms = _params(B, n, 4.0, prm)
    L = B.lib()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.boids_step_noalloc(C.byref(prms), dummy, dummy, dummy, dummy, None)
    assert rc == -1
    msg = L.boids_last_error().decode()
    assert "scratch" in msg and str(32 << 20) in msg


def _crowded_state(O, n, field, crowd, radius, seed):
    """A uniform flock with `crowd` of its boids packed in a ball of the
    given radius at the field's centre: that cell's 27-cell neighbourhood
    holds more candidates than the CTA-per-cell kernel's shared list, which
    this entry point (no id windows) leaves to the thread-per-boid kernel's
    repeated passes."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, field, (n, 3))
    d = rng.normal(size=(crowd, 3))
    d *= (radius * rng.uniform(0, 1, (crowd, 1)) ** (1 / 3)) / np.linalg.norm(d, axis=1, keepdims=True)
    pos[:crowd] = field / 2 + d
    v = rng.normal(size=(n, 3))
    v *= rng.uniform(0.001, 0.005, (n, 1)) / np.linalg.norm(v, axis=1, keepdims=True)
    return pos.astype(np.float32).reshape(-1), v.astype(np.float32).reshape(-1)


def _noalloc(B, prms, pos, vel, torch):
    dev = torch.device("cuda", 0)
    a_pos = torch.from_numpy(pos.copy()).to(dev)
    a_vel = torch.from_numpy(vel.copy()).to(dev)
    b_pos = torch.empty_like(a_pos)
    b_vel = torch.empty_like(a_vel)
    L = B.lib()
    rc = L.boids_step_noalloc(C.byref(prms), a_pos.data_ptr(), a_vel.data_ptr(),
                              b_pos.data_ptr(), b_vel.data_ptr(), None)
    assert rc == 0, L.boids_last_error().decode()
    torch.cuda.synchronize()
    return b_pos.cpu().numpy(), b_vel.cpu().numpy()


def test_noalloc_crowded_cell_matches_oracle(boids_lib, oracle_mod):
    """A cell whose neighbourhood is over 1024 candidates, three calls in a
    row, each against the oracle's update of the same state."""
    torch = pytest.importorskip("torch")
    B, O = boids_lib, oracle_mod
    n, field = 8192, 0.8
    prm = O.MARUN2019
    pos, vel = _crowded_state(O, n, field, 3000, 0.025, 5)
    p = make_params(O, n, field, prm)
    prms = _params(B, n, field, prm)
    port = O.GridPort(p, pos.copy())
    op, ov = pos.copy(), vel.copy()
    for call in range(3):
        gp, gv = _noalloc(B, prms, pos, vel, torch)
        port.step(op, ov, 1)
        assert_bits_equal(gp, op, "positions, call %d" % (call + 1))
        assert_bits_equal(gv, ov, "velocities, call %d" % (call + 1))
        pos, vel = gp, gv
    c, _ = O.neighbor_sets(p, op, ov)
    assert c[:, 0].max() > 1024  # the crowd is still one neighbourhood


def test_noalloc_alternating_parameter_sets_match_handles(boids_lib, oracle_mod):
    """Two flocks with different parameters stepped in turn (the step
    constants of both are kept between calls), on a gathered state, against
    one handle each."""
    torch = pytest.importorskip("torch")
    B, O = boids_lib, oracle_mod
    n, field = 16384, 1.0
    prm_a = O.MARUN2019
    prm_b = dict(O.MARUN2019, vmax=0.004, coh=(0.045, 0.5, 0.01))
    p = make_params(O, n, field, prm_a)
    pos0, vel0 = O.init_state(p, "random_uniform", True, 31)
    O.GridPort(p, pos0).step(pos0, vel0, 150)  # gathered
    runs = {}
    for name, prm in (("a", prm_a), ("b", prm_b)):
        sim = make_sim(B, "grid", n, field, prm, record_forces=False)
        sim.set_state(pos0, vel0)
        traj = []
        for _ in range(3):
            sim.update(1)
            traj.append(tuple(x.reshape(-1).copy() for x in sim.state()))
        sim.close()
        runs[name] = (prm, traj, [pos0.copy(), vel0.copy()])
    for call in range(3):
        for name in ("a", "b"):
            prm, traj, st = runs[name]
            gp, gv = _noalloc(B, _params(B, n, field, prm), st[0], st[1], torch)
            assert_bits_equal(gp, traj[call][0], "flock %s positions, call %d" % (name, call + 1))
            assert_bits_equal(gv, traj[call][1], "flock %s velocities, call %d" % (name, call + 1))
            st[0], st[1] = gp, gv
