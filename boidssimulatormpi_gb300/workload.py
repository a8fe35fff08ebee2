"""Runs the standard workloads of this package, for profiling and timing.

    python -m boidssimulatormpi_gb300.workload --boids 1048576 --presteps 1000 --steps 2 \\
        [--state-file s.npz] [--tuning 12,4,192,384] [--engine grid|allpairs]
    python -m boidssimulatormpi_gb300.workload --ensemble 256 --steps 100

Single flock: N boids at the reference density (16384 per unit volume, F =
(N/16384)^(1/3)), settings/marun2019.ini parameters, random_uniform with
srand48(12345), `presteps` untimed updates (the state after them can be
saved to and reloaded from --state-file, so a profiler can capture only the
updates of interest), then `steps` updates timed with synchronised wall
clock.  Ensemble: the batched sweep of boids_ensemble_* (N log-uniform in
[2^10, 2^16], factors U[0.7, 1.3] on radii, weights and vmax); its states
after `presteps` can be saved and reloaded the same way.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

MARUN2019 = dict(sep=(0.01, 0.5, 0.002), ali=(0.05, 0.3333333333333333, 0.06),
                 coh=(0.05, 0.5, 0.008), vmax=0.005, vmin=0.001)


def single(a):
    from . import BoidSimulation
    m = MARUN2019
    n = a.boids
    F = a.field or (n / 16384.0) ** (1.0 / 3.0)
    sim = BoidSimulation(a.engine, allpairs_kernels=a.allpairs_kernels)
    sim.setup(n, F, *m["sep"], *m["ali"], *m["coh"], m["vmax"], m["vmin"], "random_uniform", a.seed)
    if a.tuning:
        sim.set_tuning(*[int(x) for x in a.tuning.split(",")])
    if a.state_file and os.path.exists(a.state_file):
        d = np.load(a.state_file)
        sim.set_state(d["pos"], d["vel"])
    else:
        sim.init()
        sim.update(a.presteps)
        if a.state_file:
            p, v = sim.state()
            np.savez(a.state_file, pos=p, vel=v)
    sim.synchronize()
    t0 = time.perf_counter()
    sim.update(a.steps)
    sim.synchronize()
    dt = time.perf_counter() - t0
    print("N=%d F=%g presteps=%d: %d steps %.3f ms/step (%.3e boid-steps/s)"
          % (n, F, a.presteps, a.steps, dt * 1e3 / max(1, a.steps), n * a.steps / max(dt, 1e-12)))
    sim.close()


def ensemble(a):
    from . import Ensemble, INIT_RANDOM_UNIFORM, flock_params
    rng = np.random.default_rng(a.seed)
    m = MARUN2019
    flocks, total = [], 0
    for i in range(a.ensemble):
        n = int(round(2 ** rng.uniform(10, 16)))
        f = rng.uniform(0.7, 1.3, 7)
        F = (n / 16384.0) ** (1.0 / 3.0)
        sep = (m["sep"][0] * f[0], m["sep"][1], m["sep"][2] * f[3])
        ali = (m["ali"][0] * f[1], m["ali"][1], m["ali"][2] * f[4])
        coh = (m["coh"][0] * f[2], m["coh"][1], m["coh"][2] * f[5])
        flocks.append((flock_params(n, F, sep, ali, coh, m["vmax"] * f[6], m["vmin"]), INIT_RANDOM_UNIFORM,
                       a.seed + i))
        total += n
    ens = Ensemble(flocks)
    if a.state_file and os.path.exists(a.state_file):
        ens.init()  # then replaced flock by flock
        d = np.load(a.state_file)
        for f in range(a.ensemble):
            ens.set_state(f, d["pos%d" % f], d["vel%d" % f])
    else:
        ens.init()
        ens.step(a.presteps)
        if a.state_file:
            st = {}
            for f in range(a.ensemble):
                st["pos%d" % f], st["vel%d" % f] = ens.state(f)
            np.savez(a.state_file, **st)
    ens.synchronize()
    t0 = time.perf_counter()
    ens.step(a.steps)
    ens.synchronize()
    dt = time.perf_counter() - t0
    print("ensemble of %d flocks, %d boids: %d steps %.3f ms/step (%.3e boid-steps/s)"
          % (a.ensemble, total, a.steps, dt * 1e3 / max(1, a.steps), total * a.steps / max(dt, 1e-12)))
    ens.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--boids", type=int, default=1 << 20)
    ap.add_argument("--field", type=float, default=0.0, help="0: keep the reference density")
    ap.add_argument("--presteps", type=int, default=0)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--engine", choices=["grid", "allpairs"], default="grid")
    ap.add_argument("--allpairs-kernels", action="store_true", help="all-pairs engine on its own N^2 kernels")
    ap.add_argument("--state-file", default="")
    ap.add_argument("--tuning", default="", help="dense_min,defer_min,cand_defer,lone_cand")
    ap.add_argument("--ensemble", type=int, default=0, help="flocks (0: a single flock)")
    a = ap.parse_args(argv)
    if a.ensemble:
        ensemble(a)
    else:
        single(a)


if __name__ == "__main__":
    sys.exit(main())
