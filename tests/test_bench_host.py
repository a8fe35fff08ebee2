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
