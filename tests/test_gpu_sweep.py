"""Parameter sweeps (boidssimulatormpi_gb300.sweep) on the GPU.

* the screened sweep's values are the plain simulation's values for the
  points it picks: the simulation decides every reported value;
* what the trained network gains over the method without it: with the same
  number of re-simulated points, the surrogate's pick recovers far more of the
  plain sweep's top set of a statistic that depends on the parameters
  (nearest-neighbour distance) than points chosen blind to the statistic (at
  random, or spread over the parameter box by a Latin hypercube), seeds fixed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_BOIDS, STEPS = 1024, 40


@pytest.fixture(scope="module")
def sweep_runs(boids_lib):
    from boidssimulatormpi_gb300 import sweep as S
    ut = S.latin_hypercube(256, seed=1)
    us = S.latin_hypercube(512, seed=2)
    st_t, _ = S.simulate(ut, N_BOIDS, STEPS)
    st_s, _ = S.simulate(us, N_BOIDS, STEPS)
    sc = S.Screen(hidden=256, seed=5)
    loss, _ = sc.fit(ut, st_t, epochs=200)
    yield S, ut, us, st_t, st_s, sc, loss
    sc.close()


def test_screened_values_are_simulated_values(sweep_runs):
    S, ut, us, st_t, st_s, sc, loss = sweep_runs
    assert np.isfinite(loss)
    pick, st_pick, pred, _, _ = S.screened_sweep(sc, us, 0.05, N_BOIDS, STEPS, objective=2)
    assert pick.size == round(0.05 * 512)
    # the same point, parameters and seed give the same flock (bit-identical
    # trajectory); the FP64 sums differ only in the order of their atomic adds
    assert np.allclose(st_pick, st_s[pick], rtol=1e-12, atol=1e-15)
    assert np.array_equal(st_pick[:, 3], st_s[pick, 3])
    # the nearest-neighbour distance is a smooth function of the parameters
    assert np.corrcoef(pred[:, 2], st_s[:, 2])[0, 1] > 0.8


FRAC, OVERSAMPLE = 0.05, 2
RECALL_MIN = 0.75   # the screened pick's recall of the top 5 % (26 of 512 points)
MARGIN = 0.4        # ... above the best blind pick of the same size over five seeds


def test_network_gain_over_selection_without_it(sweep_runs):
    S, ut, us, st_t, st_s, sc, loss = sweep_runs
    o = 2  # nearest-neighbour distance
    truth = S.top(st_s[:, o], FRAC)
    pick = S.top(sc.predict(us)[:, o], FRAC * OVERSAMPLE)
    screened = S.recall(pick, truth)
    blind = [S.blind_recalls(us, truth, pick.size, seed=sd) for sd in range(5)]
    best_blind = max(max(b.values()) for b in blind)
    mean_blind = float(np.mean([v for b in blind for v in b.values()]))
    print("recall of the top %d: screened %.3f, blind best %.3f mean %.3f (budget %d of %d)"
          % (truth.size, screened, best_blind, mean_blind, pick.size, len(us)))
    assert screened >= RECALL_MIN
    assert screened >= best_blind + MARGIN
