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
  the plain simulation remains the measure of the surrogate's error.

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
             retune: bool = True) -> tuple[np.ndarray, float]:
    """Order statistics (polarization, milling, NN distance, largest cluster)
    of every point after `steps` updates, and the seconds the GPU spent
    (create/init excluded, synchronised wall time of the steps, a retuning of
    the dense-cell thresholds a quarter of the way in, and the statistics)."""
    u = np.atleast_2d(u)
    stats = np.empty((u.shape[0], 4))
    gpu_s = 0.0
    for c0 in range(0, u.shape[0], chunk):
        ens = Ensemble(flocks(u[c0:c0 + chunk], n_boids, seed))
        ens.init()
        ens.synchronize()
        t0 = time.perf_counter()
        q = steps // 4 if retune and steps >= 200 else 0
        if q:
            ens.step(q)
            ens.autotune(2)
        ens.step(steps - q)
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


# ---------------------------------------------------------------- selection without the network
#
# What the same re-simulation budget buys without the surrogate: k sweep
# points chosen blind to the statistic (at random, or spread over the
# parameter box by a Latin hypercube), or ranked by a least-squares linear
# model fitted to the same training runs.

def random_subset(n: int, k: int, seed: int = 0) -> np.ndarray:
    """k distinct indices of n, uniformly at random."""
    return np.random.default_rng(seed).choice(n, size=min(k, n), replace=False)


def lhs_subset(u: np.ndarray, k: int, seed: int = 0) -> np.ndarray:
    """k distinct points of u spread over the unit cube: for each point of a
    fresh k-point Latin hypercube, the nearest point of u not taken yet."""
    u = np.asarray(u)
    design = latin_hypercube(min(k, len(u)), u.shape[1], seed=seed)
    free = np.ones(len(u), bool)
    out = []
    for x in design:
        d = ((u - x) ** 2).sum(1)
        d[~free] = np.inf
        i = int(np.argmin(d))
        free[i] = False
        out.append(i)
    return np.array(out, dtype=np.int64)


def linear_predict(u_train: np.ndarray, y_train: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Least-squares affine model of the statistics on the parameters."""
    a = np.c_[np.asarray(u_train), np.ones(len(u_train))]
    w, *_ = np.linalg.lstsq(a, np.asarray(y_train), rcond=None)
    return np.c_[np.asarray(u), np.ones(len(u))] @ w


def blind_recalls(us: np.ndarray, truth: np.ndarray, k: int, seed: int = 0) -> dict:
    """Recall of the true top set by k points chosen without the network."""
    return {"random": recall(random_subset(len(us), k, seed), truth),
            "latin_hypercube": recall(lhs_subset(us, k, seed), truth)}


def run(n_boids=2048, steps=300, n_train=1024, n_sweep=8192, frac=0.02, oversample=(1, 2, 4), epochs=300,
        seed=12345, noise_points=64):
    """Plain sweep vs surrogate-screened sweep on the same Latin hypercube;
    returns a dict of times, the surrogate's error, and the recall of the
    plain sweep's top `frac` set for each statistic."""
    ut = latin_hypercube(n_train, seed=1)
    us = latin_hypercube(n_sweep, seed=2)
    st_train, gpu_train = simulate(ut, n_boids, steps, seed)
    st_plain, gpu_plain = simulate(us, n_boids, steps, seed)
    # the statistics' own spread from the initial placement alone
    st_other, _ = simulate(us[:noise_points], n_boids, steps, seed + 1)
    sc = Screen()
    loss, fit_s = sc.fit(ut, st_train, epochs=epochs)
    t0 = time.perf_counter()
    pred = sc.predict(us)
    infer_s = time.perf_counter() - t0
    lin = linear_predict(ut, st_train, us)
    out = {"n_boids": n_boids, "steps": steps, "train_points": n_train, "sweep_points": n_sweep, "frac": frac,
           "gpu_s": {"train_simulations": gpu_train, "plain_sweep": gpu_plain, "fit": fit_s, "inference": infer_s},
           "fit_loss": loss, "objectives": {}}
    for o, name in enumerate(OBJECTIVES):
        truth = top(st_plain[:, o], frac)
        res = {"corr": float(np.corrcoef(pred[:, o], st_plain[:, o])[0, 1]),
               "linear_corr": float(np.corrcoef(lin[:, o], st_plain[:, o])[0, 1]),
               "rmse": float(np.sqrt(np.mean((pred[:, o] - st_plain[:, o]) ** 2))),
               "spread": float(st_plain[:, o].std()),
               "seed_noise": float((st_other[:, o] - st_plain[:noise_points, o]).std() / np.sqrt(2)),
               "recall": {}}
        for m in oversample:
            pick = top(pred[:, o], frac * m)
            _, sim_s = simulate(us[pick], n_boids, steps, seed)
            res["recall"]["x%d" % m] = {"recall": recall(pick, truth), "resimulated": int(pick.size),
                                        "gpu_s": infer_s + sim_s,
                                        "fraction_of_plain": (infer_s + sim_s) / gpu_plain,
                                        "without_network": dict(blind_recalls(us, truth, pick.size, seed=m),
                                                                linear_model=recall(top(lin[:, o], frac * m),
                                                                                    truth))}
        out["objectives"][name] = res
    sc.close()
    return out


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="plain vs surrogate-screened parameter sweep")
    ap.add_argument("--boids", type=int, default=2048)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--train", type=int, default=1024)
    ap.add_argument("--sweep", type=int, default=8192)
    ap.add_argument("--frac", type=float, default=0.02)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default="", help="also write the record to this file")
    a = ap.parse_args()
    rec = run(a.boids, a.steps, a.train, a.sweep, a.frac, epochs=a.epochs)
    print(json.dumps(rec))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rec, f, indent=1)
