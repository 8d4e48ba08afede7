"""bench.py's host-side helpers, on the CPU: the clock record taken with nvidia-smi during
the timed launches (median SM clock over loaded samples, the maximum clock, the throttle
reasons that were active) and the HBM roofline denominator."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _clocks_from(rows, monkeypatch):
    monkeypatch.setattr(bench.subprocess, "Popen", lambda *a, **k: (_ for _ in ()).throw(OSError("no nvidia-smi")))
    c = bench.Clocks(0)
    assert c.p is None
    c.f.write("\n".join(rows) + "\n")
    return c.stop()


def test_clock_record_under_load(monkeypatch):
    na = "Not Active"
    rows = [f"0, 345, 2070, 110.0, 0x0, {na}, {na}, {na}, {na}",          # idle before the launches
            f"0, 2070, 2070, 900.5, 0x0, {na}, {na}, {na}, {na}",
            f"0, 2055, 2070, 1200.0, 0x4, {na}, {na}, {na}, Active",     # power cap: kept, noted
            f"0, 2070, 2070, 950.0, 0x0, {na}, {na}, {na}, {na}"]
    r = _clocks_from(rows, monkeypatch)
    assert r["sm_max_mhz"] == 2070
    assert r["sm_mhz"] == 2070            # the idle sample is not "under load"
    assert r["reasons"] == ["sw_power_cap"]
    assert r["samples"] == 4


def test_clock_record_reports_slowdowns(monkeypatch):
    na = "Not Active"
    rows = [f"0, 1500, 2070, 1300.0, 0x8, Active, {na}, Active, {na}",
            f"0, 1480, 2070, 1310.0, 0x8, Active, {na}, {na}, {na}"]
    r = _clocks_from(rows, monkeypatch)
    assert r["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert r["sm_mhz"] == pytest.approx(1490)


def test_clock_record_without_samples(monkeypatch):
    r = _clocks_from([], monkeypatch)
    assert r == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_hbm_peak_denominator():
    peak, kind = bench.hbm_peak()
    assert kind in ("measured", "fallback")
    assert peak > 1000
    if kind == "fallback":
        assert peak == 6800.0


def test_memory_workload_is_skipped_without_host_memory(monkeypatch):
    """The 2.74e9-rating set-up needs ~60 GB of host memory: with too little free the bench
    records why and generates nothing (no library call is made)."""
    monkeypatch.setattr(bench, "host_mem_available_gb", lambda: 20.0)
    out = bench.memory_workload_run(None, 0)
    assert "skipped" in out and "generate_s" not in out
    assert bench.host_mem_available_gb.__call__() == 20.0


def test_host_memory_reading():
    assert bench.host_mem_available_gb() >= 0.0
