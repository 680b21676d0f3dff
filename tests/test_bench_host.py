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


class _FakeNvml:
    """Stands in for libnvidia-ml: a fixed sequence of (SM clock, reasons) readings."""

    def __init__(self, readings, sm_max=2070):
        self.readings = list(readings)
        self.sm_max = sm_max
        self.k = 0
        self.shutdown = False

    def nvmlInit_v2(self):
        return 0

    def nvmlShutdown(self):
        self.shutdown = True
        return 0

    def nvmlDeviceGetHandleByIndex_v2(self, index, handle):
        return 0

    def nvmlDeviceGetMaxClockInfo(self, h, kind, out):
        out._obj.value = self.sm_max
        return 0

    def nvmlDeviceGetClockInfo(self, h, kind, out):
        if self.k >= len(self.readings):
            return 999                      # no more readings: the sample is skipped
        out._obj.value = self.readings[self.k][0]
        return 0

    def nvmlDeviceGetCurrentClocksEventReasons(self, h, out):
        if self.k >= len(self.readings):
            return 999
        out._obj.value = self.readings[self.k][1]
        self.k += 1
        return 0


def test_nvml_clock_record(monkeypatch):
    """The NVML sampler (every 2 ms): median SM clock, max clock, and the reason bits
    that were set during the timed region."""
    import bench

    fake = _FakeNvml([(2070, 0x0), (1995, 0x4), (2040, 0x0), (1500, 0x40)])
    with bench.NvmlClockSampler(0, lib=fake) as clk:
        t = time.monotonic()
        while fake.k < 4 and time.monotonic() - t < 10:
            time.sleep(0.005)
    s = clk.summary()
    assert s["samples"] == 4 and s["sm_mhz"] == 2017.5 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert fake.shutdown


def test_nvml_clock_record_without_gpu():
    import bench

    s = bench.NvmlClockSampler(-1)
    assert not s.ok and s.summary()["samples"] == 0
