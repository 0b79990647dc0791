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
    # clocks.sm, clocks.max.sm, power.draw, hw_slowdown, hw_thermal_slowdown,
    # sw_thermal_slowdown, sw_power_cap (nvidia-smi csv, no units)
    c.samples = [
        ["2070", "2070", "900.1", "Not Active", "Not Active", "Not Active", "Active"],
        ["1980", "2070", "950.0", "Active", "Not Active", "Not Active", "Not Active"],
        ["2070", "2070", "910.4", "Not Active", "Not Active", "Not Active", "Not Active"],
        ["[N/A]", "2070", "0", "Not Active", "Not Active", "Not Active", "Not Active"],  # unreadable row
    ]
    s = c.stop()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert s["samples"] == 3


def test_clock_summary_without_samples():
    s = bench.ClockSampler(0).stop()
    assert s == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_peaks_measured_file_and_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6782.4, "bf16_tflops": 1900.0}))
    assert bench.peaks() == (6782.4, "measured")


def test_resolve_traffic_from_the_committed_summary():
    t = bench.resolve_traffic(1.0)
    assert isinstance(t, int) and 50e6 < t < 400e6
    assert bench.resolve_traffic(0.5) is None
