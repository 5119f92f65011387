"""Host logic of bench.py (no GPU): the clock sampler keeps only the
readings whose query overlapped the timed region, and reports the median
SM clock and every throttle reason seen; the memory-side roofline figures
follow from the traffic and the kernel time; the reference arm prints one
JSON line with the contract's keys."""
import json
import os
import subprocess
import sys
import time

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _fake_smi(tmp_path, line, delay=0.02):
    p = tmp_path / "nvidia-smi"
    p.write_text("#!/bin/sh\nsleep %g\necho \"%s\"\n" % (delay, line))
    p.chmod(0o755)
    return str(tmp_path)


def test_clock_sampler_overlap(tmp_path, monkeypatch):
    d = _fake_smi(tmp_path, "2070, 2070, 0x0, Not Active, Not Active, Not Active, Active")
    monkeypatch.setenv("PATH", d + os.pathsep + os.environ.get("PATH", ""))
    c = bench.ClockSampler()
    c.start()
    time.sleep(0.3)
    out = c.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    assert out["samples"] >= 2 and 0.25 < out["region_s"] < 1.0


def test_clock_sampler_short_region_keeps_nearest(tmp_path, monkeypatch):
    d = _fake_smi(tmp_path, "1500, 2070, 0x0, Active, Not Active, Not Active, Not Active", delay=0.05)
    monkeypatch.setenv("PATH", d + os.pathsep + os.environ.get("PATH", ""))
    c = bench.ClockSampler()
    c.start()
    out = c.stop()
    assert out["samples"] == 1 and out["sm_mhz"] == 1500.0
    assert out["reasons"] == ["hw_slowdown"]


def test_clock_sampler_without_nvidia_smi(monkeypatch, tmp_path):
    monkeypatch.setenv("PATH", str(tmp_path))
    c = bench.ClockSampler()
    c.start()
    out = c.stop()
    assert out["sm_mhz"] is None and out["reasons"] == ["nvidia-smi unavailable"]


def test_clock_summary_without_max_clock():
    # readings whose max-clock field is not a number (or that are short)
    out = bench.summarize_clocks([["1980", "[N/A]", "0x0"], ["1990"]])
    assert out["sm_mhz"] == 1990.0 and out["sm_max_mhz"] is None and out["samples"] == 2


def test_hbm_side():
    out = bench.hbm_side(1.0e9, 1.0)       # 1 GB in 1 ms
    assert abs(out["dram_gbs"] - 1000.0) < 1e-9
    assert abs(out["frac_of_hbm"] - 1000.0 / out["hbm_peak_gbs"]) < 1e-12
    assert bench.hbm_side(None, 1.0) == {} and bench.hbm_side(1.0, 0.0) == {}


@pytest.mark.timeout(600)
def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["value"] > 0
    assert d["unit"] == "atom-steps/s" and d["config"]["jobs"] == 2048 and d["config"]["step_scale"] == 1.0
    assert d["warmup"] == 3 and d["steps"] == 1 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_ttm_cpu_port_runs():
    """The TTM line's CPU baseline (the oracle port's full symplectic-Euler
    step with the turi fields, solver and friction term on the 800 000-atom
    slab) runs and reports a positive rate."""
    v, k = bench.cpu_port_ttm(2, target_s=0.1, max_steps=1)
    assert v > 0 and k == 1
