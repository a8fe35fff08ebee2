"""The C++ adapter (include/boids_compat) on the GPU: oracle/ref_driver.cpp,
the driver through which the tests run the reference engine, linked against
the adapter instead of src/boid_simulation_grid.cpp, gives the oracle's bits
for init, update, get and get_force, and for a state written through the
public boids[] array and rebinned (the reference's own rebinning hooks)."""
import numpy as np
import pytest

from conftest import assert_bits_equal, make_params
from test_compat import build_adapter_driver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adapter_lib(boids_lib, tmp_path_factory):
    return build_adapter_driver(boids_lib, str(tmp_path_factory.mktemp("compat") / "libref_gb300.so"))


@pytest.mark.parametrize("n,field,sname,init,steps", [
    (4096, 0.63, "MARUN2019", "random_uniform", 20),
    (1000, 1.0, "TEST_INI", "test", 30),
])
def test_adapter_trajectory_equals_oracle(oracle_mod, adapter_lib, n, field, sname, init, steps):
    O = oracle_mod
    p = make_params(O, n, field, getattr(O, sname))
    eng = O.RefEngine("grid", p, init, 4242, lib_path=adapter_lib)
    eng.init()
    pos, vel = O.init_state(p, init, seeded=True, seed=4242)
    gp, gv = eng.state()
    assert_bits_equal(gp, pos, "init positions")
    assert_bits_equal(gv, vel, "init velocities")
    port = O.GridPort(p, pos)
    for _ in range(steps):  # one update() per call, as the reference's frame loop does
        eng.update(1)
    f = port.step(pos, vel, steps, forces=True)
    gp, gv = eng.state()
    assert_bits_equal(gp, pos, "positions after %d updates" % steps)
    assert_bits_equal(gv, vel, "velocities after %d updates" % steps)
    assert_bits_equal(eng.forces(), f, "get_force after %d updates" % steps)
    eng.close()


def test_adapter_state_written_through_boids_array(oracle_mod, adapter_lib):
    O = oracle_mod
    n, field = 8192, 0.8
    p = make_params(O, n, field, O.MARUN2019)
    pos, vel = O.init_state(p, "random_uniform", True, 17)
    O.GridPort(p, pos).step(pos, vel, 80)  # a gathered state
    eng = O.RefEngine("grid", p, "random_uniform", 1, lib_path=adapter_lib)
    eng.init()
    eng.set_state(pos, vel)  # writes boids[] and rebins
    eng.update(1)
    f = O.GridPort(p, pos).step(pos, vel, 1, forces=True)
    gp, gv = eng.state()
    assert_bits_equal(gp, pos, "positions")
    assert_bits_equal(gv, vel, "velocities")
    assert_bits_equal(eng.forces(), f, "forces")
    eng.close()
