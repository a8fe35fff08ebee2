"""bench.py's host-side helpers, no GPU: the clock record it attaches to its
line (median SM clock under load, the maximum, and every throttle reason that
was active in any sample)."""
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_clock_summary_reports_median_max_and_active_reasons():
    import bench
    c = bench.ClockSampler(0)
    c.lines = [
        "0, 2070, 2070, 905.12, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1399.80, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1210.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "[N/A]",  # a malformed sample is skipped
    ]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    c.lines.append("0, 1500, 2070, 700.00, 0x0000000000000048, Active, Not Active, Active, Not Active")
    s = c.summary()
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 2025.0 and s["samples"] == 4


def test_clock_summary_without_samples():
    import bench
    c = bench.ClockSampler(0)
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def _args(**kw):
    import argparse
    d = dict(n=2048, field=0.5, seed=777, engine="grid", allpairs_kernels=False, cpu_sample_steps=2)
    d.update(kw)
    return argparse.Namespace(**d)


def test_both_arms_report_the_same_config(monkeypatch):
    import bench
    a = _args()
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    c = bench.workload(a)
    assert c == bench.workload(a) and c["parallelism"] == "single GPU" and c["kernels"] == "grid"
    assert "flushed" in c["l2"]
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.workload(a)["parallelism"] == "replicas"


def test_cpu_baseline_parity_flag_counts_mismatches(oracle_mod):
    """The in-bench parity check: the CPU baseline's updates from the timed
    state against the GPU's, value by value (here the oracle stands in for
    the GPU, once exact and once with two values planted wrong)."""
    import numpy as np
    import bench
    O = oracle_mod
    a = _args()
    p = O.params(a.n, a.field, O.MARUN2019["sep"], O.MARUN2019["ali"], O.MARUN2019["coh"],
                 O.MARUN2019["vmax"], O.MARUN2019["vmin"])
    pos0, vel0 = O.init_state(p, "random_uniform", True, a.seed)
    pos, vel = pos0.copy(), vel0.copy()
    O.GridPort(p, pos).step(pos, vel, a.cpu_sample_steps)
    out = bench.cpu_baseline_sample(a, pos0, vel0, (pos, vel))
    assert out["parity"]["result"] == "bit-exact" and out["parity"]["mismatched_values"] == 0
    assert out["parity"]["values"] == 6 * a.n and out["single_thread"]["cores"] == 1
    assert out["value"] > 0 and out["single_thread"]["value"] > 0
    bad = pos.copy()
    bad[5] = np.nextafter(bad[5], np.float32(2))
    badv = vel.copy()
    badv[7] = -badv[7]
    out = bench.cpu_baseline_sample(a, pos0, vel0, (bad, badv))
    assert out["parity"]["result"] == "MISMATCH" and out["parity"]["mismatched_values"] == 2
