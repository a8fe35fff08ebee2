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
