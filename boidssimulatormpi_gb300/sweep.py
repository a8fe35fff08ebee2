"""Parameter sweeps of the boid update, plain and surrogate-screened.

A sweep point is a vector of the eight rule parameters
(r_sep, r_ali, r_coh, c_sep, c_ali, c_coh, vmin, vmax), each the
settings/marun2019.ini value scaled by a factor in [0.7, 1.3]; the view
angles stay fixed.  Points are simulated as flocks of one batched ensemble
(``boids_ensemble_*``: one launch per kernel per step for all flocks), all
from the same seeded initial placement, and scored by the ensemble's order
statistics after the run.

* plain sweep: every point simulated;
* screened sweep: the surrogate network (``boids_mlp_*``, BF16 tensor-core
  MLP trained on simulated points) ranks every point, and only its predicted
  top fraction is simulated, which also gives the values the sweep reports;
  the plain simulation stays the judge of the surrogate's error.

No counterpart in the reference, which runs one flock per process.
"""
from __future__ import annotations

import time

import numpy as np

from . import BoidSimulation, Ensemble, INIT_RANDOM_UNIFORM, STAT_NAMES, Surrogate, flock_params  # noqa: F401

PARAM_NAMES = ("r_sep", "r_ali", "r_coh", "c_sep", "c_ali", "c_coh", "vmin", "vmax")
# settings/marun2019.ini: sight distances, force coefficients, speed limits
BASE = np.array([0.01, 0.05, 0.05, 0.002, 0.06, 0.008, 0.001, 0.005])
ANGLES = (0.5, 0.3333333333333333, 0.5)  # separation, alignment, cohesion
LOW, HIGH = 0.7, 1.3
OBJECTIVES = STAT_NAMES[:4]


def latin_hypercube(n: int, d: int = 8, seed: int = 0) -> np.ndarray:
    """n points in [0, 1)^d, one per stratum of every axis."""
    rng = np.random.default_rng(seed)
    u = np.empty((n, d))
    for j in range(d):
        u[:, j] = (rng.permutation(n) + rng.random(n)) / n
    return u


def to_params(u: np.ndarray) -> np.ndarray:
    """Unit-cube points to parameter values (factors in [LOW, HIGH])."""
    return BASE * (LOW + (HIGH - LOW) * np.asarray(u))


def flocks(u: np.ndarray, n_boids: int, seed: int, device: int = 0):
    """Ensemble descriptions of the points u: same N, field and seed for all."""
    field = (n_boids / 16384.0) ** (1.0 / 3.0)
    out = []
    for v in to_params(u):
        sep = (v[0], ANGLES[0], v[3])
        ali = (v[1], ANGLES[1], v[4])
        coh = (v[2], ANGLES[2], v[5])
        out.append((flock_params(n_boids, field, sep, ali, coh, v[7], v[6], device), INIT_RANDOM_UNIFORM, seed))
    return out


def simulate(u: np.ndarray, n_boids: int, steps: int, seed: int = 12345, chunk: int = 8192,
             autotune: bool = True) -> tuple[np.ndarray, float]:
    """Order statistics (polarization, milling, NN distance, largest cluster)
    of every point after `steps` updates, and the seconds the GPU spent
    (create/init excluded, synchronised wall time of the steps and stats)."""
    u = np.atleast_2d(u)
    stats = np.empty((u.shape[0], 4))
    gpu_s = 0.0
    for c0 in range(0, u.shape[0], chunk):
        ens = Ensemble(flocks(u[c0:c0 + chunk], n_boids, seed))
        ens.init()
        if autotune and steps >= 64:
            ens.autotune()
        ens.synchronize()
        t0 = time.perf_counter()
        ens.step(steps)
        st = ens.stats()
        gpu_s += time.perf_counter() - t0
        stats[c0:c0 + chunk] = st[:, :4]
        ens.close()
    return stats, gpu_s


class Screen:
    """A surrogate fitted to simulated points: standardised targets, unit-cube inputs."""

    def __init__(self, hidden: int = 256, seed: int = 1):
        self.net = Surrogate(8, hidden, 4, seed=seed)
        self.mu = np.zeros(4)
        self.sd = np.ones(4)

    def fit(self, u: np.ndarray, stats: np.ndarray, epochs: int = 300, batch: int = 256, lr: float = 2e-3):
        self.mu = stats.mean(0)
        self.sd = stats.std(0) + 1e-12
        t0 = time.perf_counter()
        loss = self.net.train(np.asarray(u, np.float32), ((stats - self.mu) / self.sd).astype(np.float32),
                              epochs=epochs, batch=batch, lr=lr)
        return loss, time.perf_counter() - t0

    def predict(self, u: np.ndarray) -> np.ndarray:
        return self.net.predict(np.asarray(u, np.float32)).astype(np.float64) * self.sd + self.mu

    def close(self):
        self.net.close()


def top(values: np.ndarray, frac: float) -> np.ndarray:
    """Indices of the largest `frac` of values (at least one)."""
    k = max(1, int(round(frac * values.size)))
    return np.argsort(-values, kind="stable")[:k]


def screened_sweep(screen: Screen, u: np.ndarray, frac: float, n_boids: int, steps: int, objective: int = 0,
                   seed: int = 12345):
    """Rank every point with the surrogate, simulate its predicted top `frac`."""
    t0 = time.perf_counter()
    pred = screen.predict(u)
    infer_s = time.perf_counter() - t0
    pick = top(pred[:, objective], frac)
    stats, sim_s = simulate(u[pick], n_boids, steps, seed)
    return pick, stats, pred, infer_s, sim_s


def recall(chosen: np.ndarray, truth: np.ndarray) -> float:
    return len(set(chosen.tolist()) & set(truth.tolist())) / max(1, len(truth))
