"""bench.py's clock record on CPU: the nvidia-smi sampler against a fake
nvidia-smi (median SM clock, max clock, throttle reasons, sample count) and
its behaviour without one."""
import os
import stat
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the sampler's query: index, clocks.sm, clocks.max.sm, power.draw, reasons.active,
# hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
FAKE = """#!/bin/sh
i=0
while [ $i -lt 200 ]; do
  case $((i % 3)) in
    0) echo "0, 1980, 2070, 610.5, 0x4, Not Active, Not Active, Not Active, Active" ;;
    1) echo "0, 2010, 2070, 655.0, 0x0, Not Active, Not Active, Not Active, Not Active" ;;
    2) echo "0, 1995, 2070, 640.2, 0x0, Not Active, Not Active, Not Active, Not Active" ;;
  esac
  i=$((i + 1))
  sleep 0.05
done
"""


def _fake_smi(tmp_path, body):
    d = tmp_path / "bin"
    d.mkdir()
    exe = d / "nvidia-smi"
    exe.write_text(body)
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    return str(d)


def test_clock_sampler_parses_clocks_and_reasons(tmp_path, monkeypatch):
    pytest.importorskip("torch")
    import bench

    monkeypatch.setenv("PATH", _fake_smi(tmp_path, FAKE) + os.pathsep + os.environ["PATH"])
    c = bench.ClockSampler(0)
    c.start()
    time.sleep(0.4)
    out = c.stop()
    assert out["samples"] >= 3
    assert out["sm_max_mhz"] == 2070.0
    assert 1980.0 <= out["sm_mhz"] <= 2010.0
    assert out["reasons"] == ["sw_power_cap"]
    assert out["power_w_max"] >= 610.5


def test_clock_sampler_flags_slowdown(tmp_path, monkeypatch):
    pytest.importorskip("torch")
    import bench

    body = "#!/bin/sh\nwhile true; do echo \"0, 1200, 2070, 300.0, 0x8, Active, Active, Not Active, Not Active\"; sleep 0.05; done\n"
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, body) + os.pathsep + os.environ["PATH"])
    c = bench.ClockSampler(0)
    c.start()
    time.sleep(0.2)
    out = c.stop()
    assert out["samples"] >= 1 and out["sm_mhz"] == 1200.0
    assert out["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    pytest.importorskip("torch")
    import bench

    empty = tmp_path / "empty"
    empty.mkdir()
    monkeypatch.setenv("PATH", str(empty))
    c = bench.ClockSampler(0)
    c.start()
    out = c.stop()
    assert out == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
    assert c.path is None or not os.path.exists(c.path)  # no temporary file left behind
