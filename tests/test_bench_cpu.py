"""bench.py's reference arm (the CPU restatement timed on the host cores) runs
on a host without a GPU and prints one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line(built_lib):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "c0",
                          "--steps", "1", "--warmup", "1", "--ref-budget-s", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "steps/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "64x64 cloth" in d["config"]["workload"]


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_sampler_keeps_the_samples_of_the_timed_region():
    """Only samples stamped inside the timed region count; a region shorter than
    the sampling period takes the first sample after its start; the throttle
    reasons of the kept samples are reported."""
    import datetime
    b = _bench_module()
    now = datetime.datetime.now()

    def line(dt, sm, cap="Not Active"):
        ts = (now + datetime.timedelta(seconds=dt)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return f"{ts}, 0, {sm}, 2070, 900, 0x0, Not Active, Not Active, Not Active, {cap}"

    c = b.ClockSampler(0)
    c.lines = [line(-0.5, 345), line(0.1, 2070, "Active"), line(0.3, 2055), line(0.9, 1200)]
    c.t_start, c.t_end = now, now + datetime.timedelta(seconds=0.5)
    assert c.summary() == {"sm_mhz": 2062.5, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 2}
    c.t_end = now + datetime.timedelta(seconds=0.05)
    assert c.summary()["samples"] == 1 and c.summary()["sm_mhz"] == 2070.0
    c.lines = ["garbage", line(-0.5, 345)]
    assert c.summary()["reasons"] == ["unavailable"]
