"""Host logic of bench.py on CPU: the clock record parses nvidia-smi's CSV lines into the
median SM clock under load, the maximum clock and the throttle reasons that were active
(a fake nvidia-smi on PATH stands in for the real one)."""
import os
import stat
import sys
import time

from conftest import ROOT

sys.path.insert(0, str(ROOT))


def _fake_smi(tmp_path, lines):
    exe = tmp_path / "nvidia-smi"
    body = "".join(f"echo '{l}'\n" for l in lines)
    exe.write_text("#!/bin/sh\n" + body + "exec sleep 30\n")
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    return exe


def test_clock_record_median_max_and_reasons(tmp_path, monkeypatch):
    import bench

    na = "Not Active"
    _fake_smi(tmp_path, [
        f"0, 2070, 2070, 900.1, 0x0, {na}, {na}, {na}, {na}",
        f"0, 1980, 2070, 1390.0, 0x4, {na}, {na}, {na}, Active",
        f"0, 2010, 2070, 1200.5, 0x0, {na}, {na}, {na}, {na}",
        "garbage line",
    ])
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    with bench.ClockSampler(0) as clk:
        t = time.monotonic()
        while len(clk.lines) < 4 and time.monotonic() - t < 10:
            time.sleep(0.02)
    s = clk.summary()
    assert s == {"sm_mhz": 2010.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"],
                 "samples": 3}


def test_clock_record_flags_thermal_slowdown(tmp_path, monkeypatch):
    import bench

    na = "Not Active"
    _fake_smi(tmp_path, [f"0, 1500, 2070, 800.0, 0x40, {na}, Active, {na}, {na}"])
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    with bench.ClockSampler(0) as clk:
        t = time.monotonic()
        while not clk.lines and time.monotonic() - t < 10:
            time.sleep(0.02)
    assert clk.summary()["reasons"] == ["hw_thermal_slowdown"]


def test_clock_record_without_nvidia_smi(tmp_path, monkeypatch):
    import bench

    monkeypatch.setenv("PATH", str(tmp_path))      # no nvidia-smi anywhere
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
