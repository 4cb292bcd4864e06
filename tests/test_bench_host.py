"""Host logic of bench.py that needs no GPU: the clock sampler that records SM clocks and
throttle reasons during the timed region (driven here by a stand-in nvidia-smi that prints the
same CSV fields), and the whole-job aggregation of replica timings."""
import os
import stat
import sys
import time

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def fake_smi(tmp_path, line):
    path = tmp_path / "nvidia-smi"
    path.write_text("#!/bin/bash\nsleep 0.2\nwhile true; do echo \"%s\"; sleep 0.1; done\n" % line)
    path.chmod(path.stat().st_mode | stat.S_IXUSR)
    return str(tmp_path)


@pytest.mark.parametrize("line,reasons", [
    ("0, 2070, 2070, 850.1, 0x0, Not Active, Not Active, Not Active, Not Active", []),
    ("0, 1500, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active", ["sw_power_cap"]),
    ("0, 900, 2070, 700.0, 0x8, Active, Not Active, Not Active, Not Active", ["hw_slowdown"]),
])
def test_clock_sampler_reports_the_timed_region(tmp_path, monkeypatch, line, reasons):
    import bench
    monkeypatch.setenv("PATH", fake_smi(tmp_path, line) + os.pathsep + os.environ["PATH"])
    c = bench.ClockSampler(0)
    c.start()
    assert c.lines, "start() waits for the first sample"
    c.mark()
    time.sleep(0.55)
    out = c.stop()
    assert out["samples"] >= 2
    assert out["sm_mhz"] == float(line.split(",")[1])
    assert out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == reasons


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))
    c = bench.ClockSampler(0)
    c.start()
    c.mark()
    out = c.stop()
    assert out["sm_mhz"] is None and out["reasons"] == ["nvidia-smi unavailable"]


def test_aggregate_single_rank():
    import bench
    ms, value = bench.aggregate(100.0, 1000, 10)
    assert ms == 100.0 and value == pytest.approx(1000 * 10 / 0.1)
