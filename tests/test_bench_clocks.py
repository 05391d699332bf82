"""The benchmark's clock sampler (no GPU): samples from a stand-in nvidia-smi on PATH become
the median SM clock, the maximum clock and the throttle reasons seen."""
import os
import stat
import sys
import time


def test_clock_summary(tmp_path, monkeypatch):
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\n"
                    "echo '0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active'\n"
                    "echo '0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active'\n"
                    "echo '0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active'\n"
                    "sleep 30\n")
    fake.chmod(fake.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ["PATH"])
    monkeypatch.setenv("GBCHEM_CLOCKS_CSV", str(tmp_path / "clocks.csv"))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    with bench.Clocks(0) as c:
        time.sleep(0.5)
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    assert (tmp_path / "clocks.csv").exists()


def test_clock_summary_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    with bench.Clocks(0) as c:
        pass
    assert c.summary()["reasons"] == ["nvidia-smi unavailable"]
