"""bench.py's clock sampler against a stand-in `nvidia-smi` that prints a fixed sample every 10 ms:
it keeps only the samples taken inside the timed region and reports the median SM clock and the
throttle reasons seen there."""
import os
import stat
import sys
import time

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


@pytest.fixture
def fake_smi(tmp_path, monkeypatch):
    script = tmp_path / "nvidia-smi"
    script.write_text("#!/bin/sh\nwhile true; do echo '1980, 2070, 0x4, Not Active, Not Active, Not Active, Active'; "
                      "sleep 0.01; done\n")
    script.chmod(script.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ.get('PATH', '')}")
    return script


def test_clock_sampler_region(fake_smi):
    import bench
    with bench.ClockSampler(0, period_ms=10) as clk:
        time.sleep(0.2)
    s = clk.summary()
    assert s["sm_mhz"] == 1980.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] >= 3


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))
    with bench.ClockSampler(0, period_ms=10) as clk:
        pass
    assert clk.summary()["reasons"] == ["unsampled"]
