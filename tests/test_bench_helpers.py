"""bench.py's host-side helpers, on the CPU: the clock summary that the line's
`clocks` object comes from, the peak file with its fallback, and the resolve
stage's DRAM traffic read from the committed ncu summary."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_clock_summary_reports_median_max_and_active_reasons():
    c = bench.ClockSampler(0)
    # NVML child lines: monotonic s, SM MHz, max MHz, clock-event reason bits, power mW
    lines = ["10.000,2070,2070,4,900100",      # sw_power_cap
             "10.010,1980,2070,8,950000",      # hw_slowdown
             "10.020,2070,2070,0,910400",
             "10.030,2070,2070,64,0",          # hw_thermal_slowdown, outside the window
             "garbage"]
    c.samples = [x for x in map(bench.ClockSampler.parse_nvml, lines) if x]
    assert len(c.samples) == 4
    c.t0, c.t1 = 9.99, 10.025
    s = c.stop()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["sm_min_mhz"] == 1980.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert s["samples"] == 3
    assert s["power_w"] == 910.4


def test_clock_summary_of_nvidia_smi_lines():
    # clocks.sm, clocks.max.sm, power.draw, hw_slowdown, hw_thermal_slowdown,
    # sw_thermal_slowdown, sw_power_cap (csv, no units)
    rows = ["2070, 2070, 900.1, Not Active, Not Active, Not Active, Active",
            "1980, 2070, 950.0, Active, Not Active, Not Active, Not Active",
            "[N/A], 2070, 0, Not Active, Not Active, Not Active, Not Active"]  # unreadable row
    got = [bench.ClockSampler.parse_smi(r, 1.0) for r in rows]
    assert got[2] is None
    assert got[0][3] == ["sw_power_cap"] and got[1][3] == ["hw_slowdown"] and got[1][1] == 1980.0


def test_clock_summary_without_samples():
    s = bench.ClockSampler(0).stop()
    assert s["sm_mhz"] is None and s["sm_max_mhz"] is None and s["reasons"] == [] and s["samples"] == 0


def test_peaks_measured_file_and_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6782.4, "bf16_tflops": 1900.0}))
    assert bench.peaks() == (6782.4, "measured")


def test_resolve_traffic_from_the_committed_summary():
    t = bench.resolve_traffic(1.0)
    assert isinstance(t, int) and 50e6 < t < 400e6
    assert bench.resolve_traffic(0.5) is None
