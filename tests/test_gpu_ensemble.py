"""Batched ensembles (boids_ensemble_*) on the GPU.

* Every flock of an ensemble follows, bit for bit, the trajectory of a
  single grid-engine handle with the same parameters and seed (itself
  bit-identical to the oracle and the reference, test_gpu_parity.py),
  through the captured-graph steps, the direct steps, the statistics pass,
  a mid-run set_state and the autotuner.
* The per-flock statistics equal a numpy/scipy computation on the same
  states (FP64 sums to 1e-9 relative, link clusters exactly).
"""
import numpy as np
import pytest

from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu

MARUN = dict(sep=(0.01, 0.5, 0.002), ali=(0.05, 0.3333333333333333, 0.06),
             coh=(0.05, 0.5, 0.008), vmax=0.005, vmin=0.001)


def scaled(rng, n):
    """A flock of the ensemble sweep: the marun2019 parameters with radii,
    weights and vmax scaled by factors in [0.7, 1.3], at density 16384."""
    f = rng.uniform(0.7, 1.3, 7)
    sep = (MARUN["sep"][0] * f[0], MARUN["sep"][1], MARUN["sep"][2] * f[3])
    ali = (MARUN["ali"][0] * f[1], MARUN["ali"][1], MARUN["ali"][2] * f[4])
    coh = (MARUN["coh"][0] * f[2], MARUN["coh"][1], MARUN["coh"][2] * f[5])
    field = (n / 16384.0) ** (1.0 / 3.0)
    return field, sep, ali, coh, MARUN["vmax"] * f[6], MARUN["vmin"]


def make(B, spec):
    """spec: list of (n, field, sep, ali, coh, vmax, vmin, init_kind, seed)."""
    flocks = [(B.flock_params(n, F, sep, ali, coh, vmax, vmin), kind, seed)
              for n, F, sep, ali, coh, vmax, vmin, kind, seed in spec]
    ens = B.Ensemble(flocks)
    ens.init()
    singles = []
    for n, F, sep, ali, coh, vmax, vmin, kind, seed in spec:
        s = B.BoidSimulation("grid")
        s.setup(n, F, *sep, *ali, *coh, vmax, vmin, "test" if kind == B.INIT_TEST else "random_uniform", seed)
        s.init()
        singles.append(s)
    return ens, singles


def check_same(ens, singles, what):
    for f, s in enumerate(singles):
        ep, ev = ens.state(f)
        sp, sv = s.state()
        assert_bits_equal(ep, sp, "%s: flock %d positions" % (what, f))
        assert_bits_equal(ev, sv, "%s: flock %d velocities" % (what, f))


def spec_mixed(B, seed=7):
    rng = np.random.default_rng(seed)
    spec = []
    for i, n in enumerate([1000, 4096, 333, 20000, 1024, 7000, 600, 2500]):
        field, sep, ali, coh, vmax, vmin = scaled(rng, n)
        kind = B.INIT_TEST if i == 4 else B.INIT_RANDOM_UNIFORM
        if kind == B.INIT_TEST:  # the test placement crowds a quarter of the box
            field *= 2.0
        spec.append((n, field, sep, ali, coh, vmax, vmin, kind, 1000 + i))
    return spec


def test_flocks_match_single_handles(boids_lib):
    B = boids_lib
    ens, singles = make(B, spec_mixed(B))
    check_same(ens, singles, "init")
    ens.step(37)  # two captured graphs of 16 steps and 5 direct steps
    for s in singles:
        s.update(37)
    check_same(ens, singles, "37 steps")
    assert ens.kernel_launches() > 0


def test_statistics_pass_and_set_state_keep_parity(boids_lib):
    B = boids_lib
    spec = spec_mixed(B, seed=11)
    ens, singles = make(B, spec)
    ens.step(10)
    for s in singles:
        s.update(10)
    ens.stats()  # bins the state; the next step reuses that binning
    ens.step(21)
    for s in singles:
        s.update(21)
    check_same(ens, singles, "after stats")
    # replace flock 3's state with flock 3 of another seed
    p, v = singles[0].state()
    other = B.BoidSimulation("grid")
    n, F, sep, ali, coh, vmax, vmin, kind, seed = spec[3]
    other.setup(n, F, *sep, *ali, *coh, vmax, vmin, "random_uniform", 424242)
    other.init()
    op, ov = other.state()
    ens.set_state(3, op, ov)
    singles[3].set_state(op, ov)
    ens.step(17)
    for s in singles:
        s.update(17)
    check_same(ens, singles, "after set_state")


def test_autotune_keeps_results(boids_lib):
    B = boids_lib
    ens, singles = make(B, spec_mixed(B, seed=3))
    ens.step(40)
    for s in singles:
        s.update(40)
    t = ens.autotune(2)
    assert len(t) == 4
    check_same(ens, singles, "autotune leaves the state")
    ens.step(20)
    for s in singles:
        s.update(20)
    check_same(ens, singles, "stepping with the tuned thresholds")


def test_set_tuning_keeps_results(boids_lib):
    """boids_ensemble_set_tuning from all-dense to all-sparse thresholds: the
    trajectories stay the single handles' bit for bit."""
    B = boids_lib
    ens, singles = make(B, spec_mixed(B, seed=13))
    ens.set_tuning(1, 1, 0, 0)
    assert ens.tuning() == (1, 1, 0, 0)
    ens.step(30)
    for s in singles:
        s.update(30)
    check_same(ens, singles, "all-dense thresholds")
    ens.set_tuning(1 << 30, 1 << 30, 1 << 30, 1 << 30)
    ens.step(20)
    for s in singles:
        s.update(20)
    check_same(ens, singles, "all-sparse thresholds")


@pytest.mark.slow
def test_clustered_flocks_match(boids_lib):
    """Long enough for the flocks to gather (dense-cell kernel in use)."""
    B = boids_lib
    rng = np.random.default_rng(5)
    spec = []
    for i, n in enumerate([8192, 16384, 3000, 30000]):
        field, sep, ali, coh, vmax, vmin = scaled(rng, n)
        spec.append((n, field, sep, ali, coh, vmax, vmin, B.INIT_RANDOM_UNIFORM, 77 + i))
    ens, singles = make(B, spec)
    ens.step(400)
    for s in singles:
        s.update(400)
    check_same(ens, singles, "400 steps")


# ------------------------------------------------------------------ statistics


def np_stats(p, v, F, link, side):
    """The statistics of boids_ensemble_stats, restated with numpy/scipy."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    from scipy.spatial import cKDTree
    n = p.shape[0]
    pd, vd = p.astype(np.float64), v.astype(np.float64)
    sp = np.linalg.norm(vd, axis=1)
    vh = np.where(sp[:, None] > 0, vd / np.where(sp > 0, sp, 1)[:, None], 0)
    pol = np.linalg.norm(vh.sum(0)) / n
    th = 2 * np.pi * pd / F
    com = np.arctan2(np.sin(th).sum(0), np.cos(th).sum(0)) / (2 * np.pi) * F
    com = np.where(com < 0, com + F, com)
    r = pd - com
    r = np.where(r > F / 2, r - F, np.where(r < -F / 2, r + F, r))
    rn = np.linalg.norm(r, axis=1)
    rh = np.where(rn[:, None] > 0, r / np.where(rn > 0, rn, 1)[:, None], 0)
    mill = np.linalg.norm(np.cross(rh, vh).sum(0)) / n
    tree = cKDTree(np.mod(pd, F), boxsize=F)
    d, _ = tree.query(np.mod(pd, F), k=2)
    nn = np.minimum(d[:, 1], side).mean()
    # links: the float32 arithmetic of the kernel, pair images by minimum image
    pairs = tree.query_pairs(float(link) * 1.01, output_type="ndarray")
    i, j = pairs[:, 0], pairs[:, 1]
    F32 = np.float32(F)
    dd = []
    for a in range(3):
        dx = p[j, a] - p[i, a]
        sh = np.where(dx > F32 / 2, -F32, np.where(dx < -F32 / 2, F32, np.float32(0)))
        dd.append((p[j, a] + sh) - p[i, a])
    d2 = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]
    keep = d2 < np.float32(link) * np.float32(link)
    g = coo_matrix((np.ones(keep.sum()), (i[keep], j[keep])), shape=(n, n))
    _, lab = connected_components(g, directed=False)
    largest = np.bincount(lab).max() / n
    return pol, mill, nn, largest, com, vd.mean(0)


@pytest.mark.parametrize("steps", [0, 150])
def test_statistics_match_numpy(boids_lib, steps):
    pytest.importorskip("scipy")
    B = boids_lib
    spec = spec_mixed(B, seed=19)
    ens, singles = make(B, spec)
    ens.step(steps)
    st = ens.stats()
    for f, (n, F, sep, ali, coh, vmax, vmin, kind, seed) in enumerate(spec):
        p, v = ens.state(f)
        side = st[f, 10]
        pol, mill, nn, largest, com, mom = np_stats(p, v, F, np.float32(coh[0]), side)
        assert st[f, 0] == pytest.approx(pol, rel=1e-9, abs=1e-12)
        assert st[f, 1] == pytest.approx(mill, rel=1e-7, abs=1e-9)
        assert st[f, 2] == pytest.approx(nn, rel=2e-6)
        assert st[f, 3] == largest, (f, st[f, 3], largest)
        assert np.allclose(st[f, 4:7], com, rtol=0, atol=1e-6 * F)
        assert np.allclose(st[f, 7:10], mom, rtol=1e-9, atol=1e-13)
    # the statistics pass did not disturb the trajectories
    ens.step(5)
    for s in singles:
        s.update(steps + 5)
    check_same(ens, singles, "after statistics")
