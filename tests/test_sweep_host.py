"""The host side of the parameter sweeps (boidssimulatormpi_gb300.sweep),
no GPU: the Latin hypercube, the mapping of a sweep point onto a flock's
parameters, and the top-fraction and recall arithmetic the screened sweep is
scored with."""
import numpy as np
import pytest


def test_latin_hypercube_strata():
    from boidssimulatormpi_gb300 import sweep as S
    u = S.latin_hypercube(64, 8, seed=3)
    assert u.shape == (64, 8) and (u >= 0).all() and (u < 1).all()
    for j in range(8):
        assert sorted(np.floor(u[:, j] * 64).astype(int).tolist()) == list(range(64))
    p = S.to_params(np.zeros((1, 8)))
    assert np.allclose(p, S.BASE * S.LOW)
    assert np.array_equal(S.latin_hypercube(64, 8, seed=3), u)  # seeded


def test_sweep_point_to_flock_parameters():
    """Point coordinates (r_sep, r_ali, r_coh, c_sep, c_ali, c_coh, vmin,
    vmax) land in the matching setup fields; angles stay at marun2019's."""
    from boidssimulatormpi_gb300 import sweep as S
    import boidssimulatormpi_gb300 as B
    u = np.linspace(0.0, 0.875, 8)[None, :]
    v = S.to_params(u)[0]
    (p, kind, seed), = S.flocks(u, 2048, seed=77)
    assert kind == B.INIT_RANDOM_UNIFORM and seed == 77
    assert p.number_of_agents == 2048 and p.engine == B.ENGINE_GRID
    assert p.field_size == pytest.approx((2048 / 16384) ** (1 / 3))
    got = (p.separation_sight_distance, p.alignment_sight_distance, p.cohesion_sight_distance,
           p.separation_force_coefficient, p.alignment_force_coefficient, p.cohesion_force_coefficient,
           p.velocity_min, p.velocity_max)
    assert np.allclose(got, v, rtol=0, atol=0)
    assert (p.separation_sight_angle, p.alignment_sight_angle, p.cohesion_sight_angle) == S.ANGLES
    assert np.allclose(v / S.BASE, S.LOW + (S.HIGH - S.LOW) * u[0])


def test_top_fraction_and_recall():
    from boidssimulatormpi_gb300 import sweep as S
    vals = np.array([0.1, 0.9, 0.5, 0.9, 0.3, 0.7, 0.2, 0.8, 0.0, 0.4])
    assert S.top(vals, 0.3).tolist() == [1, 3, 7]        # largest first, ties in index order
    assert S.top(vals, 0.01).tolist() == [1]             # at least one
    assert S.recall(np.array([1, 7, 5]), S.top(vals, 0.3)) == pytest.approx(2 / 3)
    assert S.recall(np.array([], dtype=int), np.array([], dtype=int)) == 0.0


def test_selection_without_the_network():
    """The blind subsets the screened sweep is compared with: the requested
    size, distinct indices, seeded; the Latin-hypercube subset's first pick is
    the sweep point nearest the design's first point; and the linear model
    fits an affine function exactly."""
    from boidssimulatormpi_gb300 import sweep as S
    us = S.latin_hypercube(400, seed=2)
    r = S.random_subset(400, 40, seed=3)
    assert r.size == 40 and np.unique(r).size == 40 and np.array_equal(r, S.random_subset(400, 40, seed=3))
    l = S.lhs_subset(us, 40, seed=3)
    assert l.size == 40 and np.unique(l).size == 40 and np.array_equal(l, S.lhs_subset(us, 40, seed=3))
    d0 = S.latin_hypercube(40, 8, seed=3)[0]
    assert l[0] == np.argmin(((us - d0) ** 2).sum(1))
    truth = S.top(us[:, 0], 0.1)
    b = S.blind_recalls(us, truth, 40, seed=3)
    assert set(b) == {"random", "latin_hypercube"} and all(0 <= v <= 1 for v in b.values())
    y = us @ np.arange(1, 9, dtype=float)[:, None] * np.ones((1, 4)) + 0.5
    assert np.allclose(S.linear_predict(us, y, us[:5]), y[:5])
