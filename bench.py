#!/usr/bin/env python3
"""Benchmark: boid-steps/s of the per-timestep update at N=2^20 (grid, FP32).

Workload (BoidsSimulatorMPI's uniform-grid configuration): N = 2^20 boids in a
periodic cube of side F = 4.0 (the number density of 16384 boids per unit
volume), rule radii, view angles, weights and speed limits of
settings/marun2019.ini, dt = 1, initial state "random_uniform" drawn with
srand48(12345) exactly as the reference draws it.  One bench step = one
BoidSimulation::update() of all N boids.  Synthetic data: the state is
generated, no dataset is involved.

Our arm (--impl ours): the CUDA grid engine through its C ABI.  Before every
timed step a 256 MiB buffer is written to flush L2 (outside the timed
events); each step is timed with CUDA events on the engine's stream.  The
roofline's kernel time comes from the same steps repeated from the same
state with the engine's phase events on (those events between the kernels
are kept out of the headline steps).  `e2e`
times the same steps through the C ABI with host buffers: every step uploads
the state from pinned host memory, updates, and downloads the new state.

Reference arm (--impl reference): the reference's own CPU engine
(src/boid_simulation_grid.cpp, built from its sources into oracle/_ref) when
it is present, else the oracle's C port of it, on all host cores, same
workload; each step is one update() of all N boids.

Supplementary objects of our arm's line: `parity` (the GPU's updates from the
timed state against the CPU baseline's, bit for bit), `trajectory` (the
workload's whole 1000-update run from its seeded initial state, timed as one
region, with default thresholds and with one retune), `late_regime` (steps
after that run, when the flock has gathered), `allpairs` (the all-pairs
engine's N^2 kernels at N=65536, F=1.6, against the FP32 lane-issue peak),
`ensemble` (the 256-flock batched sweep) and `surrogate_sweep` (the recorded
plain vs screened sweep at 16 384 boids and 2000 updates, not timed here).

Multi-GPU (torchrun, N > 1): independent replicas, one per GPU, each with its
own seed; value = boid-steps of all ranks / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "boid-steps/s at N=2^20 (grid, FP32)"
UNIT = "boid-steps/s"
MARUN2019 = dict(sep=(0.01, 0.5, 0.002), ali=(0.05, 0.3333333333333333, 0.06),
                 coh=(0.05, 0.5, 0.008), vmax=0.005, vmin=0.001)
# algorithmic bytes per boid and step (state read + written once per pass)
RULE_BYTES = 72    # rule kernels: read pos+vel (32), write pos+vel (32), key+rank (8)
STEP_BYTES = 144   # whole step: rule kernels + scan/scatter (64 + 8)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--boids", dest="n", type=int, default=1 << 20)
    ap.add_argument("--field", type=float, default=4.0)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--engine", choices=["grid", "allpairs"], default="grid")
    ap.add_argument("--allpairs-kernels", action="store_true",
                    help="all-pairs engine: its own N^2 kernels, not the grid kernels it runs by default")
    ap.add_argument("--late-presteps", type=int, default=1000,
                    help="updates of the supplementary whole-trajectory timing, after which the "
                         "clustered regime is timed (0: skip both)")
    ap.add_argument("--cpu-sample-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ensemble-flocks", type=int, default=256,
                    help="supplementary batched-ensemble sweep (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=2000)
    return ap.parse_args()


def metric(a):
    """The headline metric, or its all-pairs counterpart under --engine allpairs."""
    if a.engine == "grid" and a.n == 1 << 20:
        return METRIC
    return "boid-steps/s at N=%d (%s, FP32)" % (a.n, "all-pairs" if a.engine == "allpairs" else "grid")


def workload(a):
    """The workload's config object, the same from both arms."""
    what = "all-pairs" if a.engine == "allpairs" else "grid"
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return {"workload": "boids %s update, N=%d, F=%g, marun2019.ini, random_uniform seed %d"
                        % (what, a.n, a.field, a.seed),
            "n": a.n, "field_size": a.field, "settings": "marun2019.ini", "dt": 1,
            "init": "random_uniform", "seed": a.seed, "engine": a.engine,
            "state": "timed from the initial state, after the warm-up steps",
            "l2": "flushed before every timed step (256 MiB write)",
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "kernels": "all pairs (N^2)" if a.engine == "allpairs" and a.allpairs_kernels else "grid"}


def dist_setup(a):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if a.impl == "ours" else "gloo"
        dist.init_process_group(backend)
        return dist.get_rank(), ws, dist
    return 0, 1, None


def reduce_over_ranks(dist, seconds, units, device=None):
    """Replicas: the slowest rank's time and the boid-steps of all ranks
    (value = units / seconds).  No collective on one rank."""
    if dist is None:
        return seconds, units
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ reference arm

def run_reference(a):
    import numpy as np
    import oracle as O
    rank, ws, dist = dist_setup(a)
    if rank != 0:
        return
    O.build()
    p = O.params(a.n, a.field, MARUN2019["sep"], MARUN2019["ali"], MARUN2019["coh"],
                 MARUN2019["vmax"], MARUN2019["vmin"])
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    if O.ref_available("grid"):
        kind = "reference"
        eng = O.RefEngine("grid", p, "random_uniform", a.seed)
        eng.init()
        step = eng.update
        sample = "src/boid_simulation_grid.cpp built from its sources (oracle/_ref), update() of all N"
    else:
        kind = "port"
        pos, vel = O.init_state(p, "random_uniform", True, a.seed)
        g = O.GridPort(p, pos)
        step = lambda k=1: g.step(pos, vel, k, threads=cores)
        sample = "oracle C port of src/boid_simulation_grid.cpp (rules in parallel, " \
                 "integration and rebinning serial as in the reference), update() of all N"
    for _ in range(a.warmup):
        step(1)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        step(1)
    dt = time.perf_counter() - t0
    value = a.n * a.steps / dt
    line = {"metric": metric(a), "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": dt * 1e3 / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": workload(a), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ ensemble sweep

def ensemble_flocks(B, count, seed):
    """The batched-ensemble sweep: each flock's N log-uniform in [2^10, 2^16],
    F keeping the density of 16384 boids per unit volume, and the marun2019
    radii, weights and vmax each scaled by a factor uniform in [0.7, 1.3]."""
    import numpy as np
    rng = np.random.default_rng(seed)
    m = MARUN2019
    flocks, total = [], 0
    for i in range(count):
        n = int(round(2 ** rng.uniform(10, 16)))
        f = rng.uniform(0.7, 1.3, 7)
        F = (n / 16384.0) ** (1.0 / 3.0)
        sep = (m["sep"][0] * f[0], m["sep"][1], m["sep"][2] * f[3])
        ali = (m["ali"][0] * f[1], m["ali"][1], m["ali"][2] * f[4])
        coh = (m["coh"][0] * f[2], m["coh"][1], m["coh"][2] * f[5])
        flocks.append((B.flock_params(n, F, sep, ali, coh, m["vmax"] * f[6], m["vmin"]),
                       B.INIT_RANDOM_UNIFORM, seed + i))
        total += n
    return flocks, total


def run_ensemble(a, B, rank, dist):
    """Sweep time of the whole ensemble for --ensemble-steps steps from its
    initial state, with the per-flock statistics at the end, on the default
    dense-cell thresholds (a retune a quarter of the way in costs more in
    trial steps than it wins)."""
    import numpy as np
    flocks, total = ensemble_flocks(B, a.ensemble_flocks, 2024 + 1000 * rank)
    ens = B.Ensemble(flocks)
    ens.init()
    ens.synchronize()
    tuning = ens.tuning()
    t0 = time.perf_counter()
    ens.step(a.ensemble_steps)
    ens.synchronize()
    dt, units = reduce_over_ranks(dist, time.perf_counter() - t0, float(total * a.ensemble_steps))
    st = ens.stats()
    launches = ens.kernel_launches()
    ens.close()
    return {"flocks": a.ensemble_flocks, "boids": total, "steps": a.ensemble_steps,
            "sweep_s": dt, "ms_per_step": dt * 1e3 / a.ensemble_steps,
            "boid_steps_per_s": units / dt, "tuning": list(tuning), "kernel_launches": launches,
            "stats_mean": {k: float(np.mean(st[:, i])) for i, k in enumerate(B.STAT_NAMES[:4])},
            "config": "N log-uniform in [2^10, 2^16], F = (N/16384)^(1/3), marun2019 radii, weights "
                      "and vmax x U[0.7, 1.3], random_uniform init, steps replayed from CUDA graphs; "
                      "timed from the initial state, default dense-cell thresholds"}


# ------------------------------------------------------------------ our arm

def cpu_baseline_sample(a, pos, vel, gpu_after=None):
    """The oracle port (or the reference engine) timed on this host: a few
    updates of all N boids from the state the timed GPU steps start from, on
    all cores, then one update on one thread.  With gpu_after = the GPU's
    state after the same number of updates from that state, the two are
    compared bit for bit (`parity`)."""
    import numpy as np
    import oracle as O
    O.build()
    p = O.params(a.n, a.field, MARUN2019["sep"], MARUN2019["ali"], MARUN2019["coh"],
                 MARUN2019["vmax"], MARUN2019["vmin"])
    cores = os.cpu_count() or 1
    k = max(1, a.cpu_sample_steps)
    p0, v0 = pos.copy(), vel.copy()
    pos, vel = pos.copy(), vel.copy()
    if O.ref_available("grid"):
        eng = O.RefEngine("grid", p, "random_uniform", a.seed)
        eng.set_state(pos, vel)
        t0 = time.perf_counter()
        eng.update(k)
        dt = time.perf_counter() - t0
        pos, vel = eng.state()
        kind = "reference"
        what = "src/boid_simulation_grid.cpp from its sources"
    else:
        g = O.GridPort(p, pos)
        t0 = time.perf_counter()
        g.step(pos, vel, k, threads=cores)
        dt = time.perf_counter() - t0
        kind = "port"
        what = "oracle C port of src/boid_simulation_grid.cpp"
    out = {"value": a.n * k / dt, "unit": UNIT, "cores": cores, "kind": kind,
           "sample": "%s, %d update() of all N=%d boids from the timed state" % (what, k, a.n)}
    # one thread, one update, from the same state (the port: the reference's
    # engine takes its thread count from OpenMP at load time)
    q, w = p0.copy(), v0.copy()
    g1 = O.GridPort(p, q)
    t0 = time.perf_counter()
    g1.step(q, w, 1, threads=1)
    dt1 = time.perf_counter() - t0
    g1.close()
    out["single_thread"] = {"value": a.n / dt1, "unit": UNIT, "cores": 1, "kind": "port",
                            "sample": "oracle C port, 1 update() of all N=%d boids on one thread" % a.n}
    if gpu_after is not None:
        gp, gv = (np.ascontiguousarray(x, np.float32).reshape(-1) for x in gpu_after)
        cp_, cv = (np.ascontiguousarray(x, np.float32).reshape(-1) for x in (pos, vel))
        bad = int(np.count_nonzero(gp.view(np.uint32) != cp_.view(np.uint32))
                  + np.count_nonzero(gv.view(np.uint32) != cv.view(np.uint32)))
        out["parity"] = {"result": "bit-exact" if bad == 0 else "MISMATCH", "mismatched_values": bad,
                         "values": int(gp.size + gv.size), "updates": k, "against": kind,
                         "what": "positions and velocities after %d updates from the timed state, "
                                 "GPU vs %s" % (k, what)}
    return out


def fp32_lane_peak(sm_mhz, sms):
    """FP32 lane-instructions per second the SMs can issue: 128 lanes per SM
    per clock."""
    return sms * 128 * sm_mhz * 1e6


def run_allpairs(a, B, local, stream, torch):
    """The all-pairs engine on its own N^2 kernels at N=65536, F=1.6 (the
    same density), the reference's src/boid_simulation.cpp configuration:
    device time per update, and the pair filter's FP32 rate against the
    lane-issue peak at the sampled SM clock (10 FP32 operations per ordered
    pair)."""
    n, field = 65536, 1.6
    m = MARUN2019
    sim = B.BoidSimulation("allpairs", device=local, allpairs_kernels=True)
    sim.setup(n, field, *m["sep"], *m["ali"], *m["coh"], m["vmax"], m["vmin"], "random_uniform", a.seed)
    sim.set_stream(stream.cuda_stream)
    sim.init()
    sim.update(3)
    steps = 60
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(steps):
            sim.update(1)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    sim.close()
    c = clk.summary()
    props = torch.cuda.get_device_properties(local)
    mhz = c["sm_mhz"] or 2070.0
    pairs = float(n) * n
    achieved = 10 * pairs / (ms / 1e3)
    peak = fp32_lane_peak(mhz, props.multi_processor_count)
    return {"n": n, "field_size": field, "kernels": "all pairs (N^2): k_ap_pairs + k_ap_accumulate",
            "steps": steps, "ms_per_step": ms, "value": n / (ms / 1e3), "unit": UNIT,
            "roofline": {"bound": "fp32_issue", "achieved": achieved / 1e12, "peak": peak / 1e12,
                         "unit": "TFLOP/s (FP32 lane operations)", "frac": achieved / peak,
                         "ops_per_pair": 10, "pairs_per_step": pairs,
                         "peak_is": "%d SMs x 128 FP32 lanes x %.0f MHz (sampled)"
                                    % (props.multi_processor_count, mhz)},
            "clocks": c}


def timed(stream, torch, fn):
    """Device time of fn()'s work on stream (CUDA events) and its wall time."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3


def run_trajectory(a, sim, stream, torch, steps, tune_at, tuning):
    """The whole trajectory of the workload: `steps` updates from the seeded
    initial state, replayed from captured graphs, timed as one region; with
    tune_at > 0 the dense-cell thresholds are retuned once after tune_at
    updates (the autotuner's trial steps are inside the timed region)."""
    sim.set_tuning(*tuning)
    sim.init()

    def run():
        if tune_at > 0:
            sim.update(tune_at)
            sim.autotune(2)
            sim.update(steps - tune_at)
        else:
            sim.update(steps)

    dev_ms, wall_ms = timed(stream, torch, run)
    return {"steps": steps, "autotune_at": tune_at if tune_at > 0 else None, "device_ms": dev_ms,
            "wall_ms": wall_ms, "ms_per_step": dev_ms / steps, "value": a.n * steps / (dev_ms / 1e3),
            "unit": UNIT, "tuning_after": list(sim.tuning())}


def run_ours(a):
    import numpy as np
    import torch
    import boidssimulatormpi_gb300 as B
    rank, ws, dist = dist_setup(a)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    m = MARUN2019
    sim = B.BoidSimulation(a.engine, device=local, allpairs_kernels=a.allpairs_kernels)
    sim.setup(a.n, a.field, *m["sep"], *m["ali"], *m["coh"], m["vmax"], m["vmin"],
              "random_uniform", a.seed + rank)
    # one non-default stream for the engine, the L2 flush and the timing events
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    sim.init()
    default_tuning = sim.tuning()
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)  # 256 MiB > L2

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    for _ in range(a.warmup):
        sim.update(1)
    barrier()
    pos0, vel0 = sim.state()  # the state the timed steps start from
    # ---- device-resident timing, L2 flushed before every step: each step is
    # one update as a user's loop runs it (its captured one-update graph)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    l0 = sim.kernel_launches()
    barrier()
    with ClockSampler(local) as clk:
        for i in range(a.steps):
            flush.zero_()
            starts[i].record(stream)
            sim.update(1)
            ends[i].record(stream)
        barrier()
    launches = sim.kernel_launches() - l0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s, units = reduce_over_ranks(dist, sum(step_ms) / 1e3, float(a.n * a.steps), dev)
    total_ms = total_s * 1e3
    value = units / total_s
    # ---- the same steps again from the same state with the engine's phase
    # events on (kernels launched one by one, CUDA events around the counting
    # sort and around the rule kernels): the rule kernels' time for the
    # roofline.  The events between kernels cost time, so the steps above
    # run without them.
    sim.set_state(pos0.reshape(-1), vel0.reshape(-1))
    sim.profile_read(True)
    sim.profile_enable(True)
    pstarts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    pends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    barrier()
    for i in range(a.steps):
        flush.zero_()
        pstarts[i].record(stream)
        sim.update(1)
        pends[i].record(stream)
    barrier()
    prof = sim.profile_read(True)
    sim.profile_enable(False)
    profiled_ms = sum(s.elapsed_time(e) for s, e in zip(pstarts, pends)) / a.steps

    # ---- end to end through the C ABI with host buffers
    hp = torch.empty(3 * a.n, dtype=torch.float32, pin_memory=True).numpy()
    hv = torch.empty(3 * a.n, dtype=torch.float32, pin_memory=True).numpy()
    for i in range(max(1, min(a.warmup, 3))):  # untimed: pinned pages touched, graphs captured
        hp[:] = pos0.reshape(-1)
        hv[:] = vel0.reshape(-1)
        sim.set_state(hp, hv)
        sim.update(1)
        sim.state(hp, hv)
    hp[:] = pos0.reshape(-1)
    hv[:] = vel0.reshape(-1)
    barrier()
    t0 = time.perf_counter()
    for i in range(a.steps):
        sim.set_state(hp, hv)
        sim.update(1)
        sim.state(hp, hv)
    barrier()
    e2e_s, e2e_units = reduce_over_ranks(dist, time.perf_counter() - t0, float(a.n * a.steps), dev)
    e2e = {"value": e2e_units / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(hp.nbytes + hv.nbytes),
           "d2h_bytes_per_step": int(hp.nbytes + hv.nbytes)}

    # ---- the GPU's updates from the timed state, for the in-bench parity check
    k_par = max(1, a.cpu_sample_steps)
    sim.set_state(pos0.reshape(-1), vel0.reshape(-1))
    sim.update(k_par)
    gpu_after = sim.state()

    # ---- supplementary: the whole trajectory, and the clustered regime at its end
    traj = late = None
    if a.late_presteps > 0:
        traj = {"default_tuning": run_trajectory(a, sim, stream, torch, a.late_presteps, 0, default_tuning),
                "autotuned": run_trajectory(a, sim, stream, torch, a.late_presteps, a.late_presteps // 4,
                                            default_tuning)}
        # the state after the whole trajectory with default thresholds
        sim.set_tuning(*default_tuning)
        sim.init()
        sim.update(a.late_presteps)
        tuned = sim.autotune()  # crowded flocks favour other dense-cell thresholds
        barrier()
        ms = []
        for i in range(a.steps):
            flush.zero_()
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            sim.update(1)
            s1.record(stream)
            s1.synchronize()
            ms.append(s0.elapsed_time(s1))
        late = {"after_steps": a.late_presteps, "ms_per_step": sum(ms) / len(ms),
                "value": a.n * len(ms) / (sum(ms) / 1e3), "unit": UNIT,
                "tuning": list(tuned), "default_tuning": list(default_tuning)}

    sim.close()
    allpairs = run_allpairs(a, B, local, stream, torch) if a.engine == "grid" and a.n == 1 << 20 else None
    ens = run_ensemble(a, B, rank, dist) if a.ensemble_flocks > 0 else None
    if rank != 0:
        return
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    rules_ms = prof["force_ms"] / max(1, prof["steps"])
    achieved = RULE_BYTES * a.n / (rules_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "rule kernels (k_grid_sparse + k_grid_dense)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_src, "traffic": None,
                "bytes_per_boid": RULE_BYTES, "rules_ms_per_step": rules_ms,
                "bin_ms_per_step": prof["bin_ms"] / max(1, prof["steps"]),
                "measured": "CUDA events around the rule kernels on the engine's stream, over the %d timed "
                            "steps repeated from the same state with phase events on (%.4f ms per step "
                            "against %.4f without them)" % (a.steps, profiled_ms, total_ms / a.steps),
                "step_frac": STEP_BYTES * a.n / (total_ms / a.steps / 1e3) / 1e9 / peak}
    tr = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tr):
        try:
            with open(tr) as f:
                tj = json.load(f)
            t = tj.get("rules_dram_bytes_per_boid")
            if t:
                roofline["traffic"] = t * a.n
            # the bound that does bind: instruction issue of the top kernel
            if tj.get("issue"):
                roofline["issue"] = tj["issue"]
        except (OSError, ValueError):
            pass
    # the surrogate-screened sweep at 16 384 boids and 2000 updates is a
    # run of its own (boidssimulatormpi_gb300.sweep, 14 minutes for 4096
    # points); its recorded result rides along, marked as such
    sweep_rec = None
    # the largest recorded sweep
    names = [x for x in ("sweep_n16384_t2000_p8192.json", "sweep_n16384_t2000.json")
             if os.path.exists(os.path.join(ROOT, "profiles", x))]
    if names:
        sw = os.path.join(ROOT, "profiles", names[0])
        try:
            with open(sw) as f:
                sj = json.load(f)
            sweep_rec = {"recorded": "profiles/%s (not timed in this run)" % names[0],
                         "n_boids": sj["n_boids"], "steps": sj["steps"], "sweep_points": sj["sweep_points"],
                         "train_points": sj["train_points"], "frac": sj["frac"],
                         "plain_sweep_gpu_s": sj["gpu_s"]["plain_sweep"],
                         "screened": {o: {m: {"recall": x["recall"], "fraction_of_plain": x["fraction_of_plain"],
                                              "random_recall": x["without_network"]["random"]}
                                          for m, x in r["recall"].items()}
                                      for o, r in sj["objectives"].items()}}
        except (OSError, ValueError, KeyError):
            sweep_rec = None
    cpu = None
    if not a.no_cpu_baseline and a.engine == "grid":
        cpu = cpu_baseline_sample(a, pos0.reshape(-1), vel0.reshape(-1), gpu_after)
    line = {"metric": metric(a), "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": total_ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": workload(a),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk.summary(),
            "parity": (cpu or {}).get("parity"),
            "trajectory": traj, "late_regime": late, "allpairs": allpairs, "ensemble": ens,
            "surrogate_sweep": sweep_rec,
            "step_ms_min_max": [min(step_ms), max(step_ms)]}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
