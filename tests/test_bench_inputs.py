"""Inputs of the benchmark line: the measured HBM peak (roofline denominator) and
the traversal kernels' DRAM bytes per frame from their committed ncu summary
(roofline.traffic), so that neither silently becomes a fallback or null; and the
summary of the clock samples taken during the timed region."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_roofline_peak_is_the_measured_one():
    peak, kind = bench.measured_peaks()
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        assert kind == "measured" and peak == float(json.load(open(p))["hbm_gbs"])
    else:
        assert kind == "fallback"


def test_profile_summary_gives_dram_bytes_per_frame():
    t = bench.profile_traffic()
    assert t is not None and 1e6 < t < 1e10
    # the summary names the kernels the bench reports and the command that made it
    text = open(bench.PROFILE_SUMMARY).read()
    assert "k_trace_closest" in text and "k_trace_shadow" in text and "ncu " in text
    assert "--clock-control none" in text


def test_clock_samples_summary():
    lines = [
        "0, 1965, 2070, 812.5, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070, 1004.1, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 998.0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 1.0, Not Active, Not Active, Not Active, Not Active",
    ]
    c = bench.ClockSampler.parse(lines)
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    hot = bench.ClockSampler.parse(["0, 1500, 2070, 1400.0, Not Active, Active, Not Active, Not Active"])
    assert hot["reasons"] == ["hw_thermal_slowdown"]
    assert bench.ClockSampler.parse([]) is None
