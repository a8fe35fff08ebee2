"""Parameter sweeps (boidssimulatormpi_gb300.sweep): the screened sweep's
values are the plain simulation's values for the points it picks (the
simulation decides every reported value), and the surrogate ranks a smooth statistic
(nearest-neighbour distance) well enough to recover most of its top set."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_screened_values_are_simulated_values(boids_lib):
    from boidssimulatormpi_gb300 import sweep as S
    ut = S.latin_hypercube(256, seed=1)
    us = S.latin_hypercube(512, seed=2)
    st_t, _ = S.simulate(ut, 1024, 40)
    st_s, _ = S.simulate(us, 1024, 40)
    sc = S.Screen(hidden=256, seed=5)
    loss, _ = sc.fit(ut, st_t, epochs=200)
    assert np.isfinite(loss)
    pick, st_pick, pred, _, _ = S.screened_sweep(sc, us, 0.05, 1024, 40, objective=2)
    assert pick.size == round(0.05 * 512)
    # the same point, parameters and seed give the same flock (bit-identical
    # trajectory); the FP64 sums differ only in the order of their atomic adds
    assert np.allclose(st_pick, st_s[pick], rtol=1e-12, atol=1e-15)
    assert np.array_equal(st_pick[:, 3], st_s[pick, 3])
    truth = S.top(st_s[:, 2], 0.05)
    assert 0.0 <= S.recall(pick, truth) <= 1.0
    # the nearest-neighbour distance is a smooth function of the parameters
    assert np.corrcoef(pred[:, 2], st_s[:, 2])[0, 1] > 0.8
    sc.close()
