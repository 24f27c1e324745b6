"""The bench's one-line JSON contract, on the small plain-512 workload: the
reference arm (CPU, the oracle) and the GPU arm print the keys a driver
reads, with consistent values."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
             "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "e2e"}


def _bench(*args, timeout=600):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _bench("--impl", "reference", "--workload", "plain-512", "--steps", "1", "--warmup", "1")
    assert BASE_KEYS <= set(d)
    assert d["impl"] == "reference" and d["unit"] == "realizations/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["config"]["workload"] == "plain-512"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["sample"] == "1 realizations of the whole 512x512 DEM"
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0


@pytest.mark.gpu
def test_gpu_arm_line():
    d = _bench("--workload", "plain-512", "--steps", "3", "--warmup", "3", "--no-exact",
               "--no-batched", "--cpu-steps", "1")
    assert BASE_KEYS <= set(d) and "impl" not in d
    assert d["value"] > 0 and d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    per_step = d["config"]["realizations_per_step"]
    assert per_step == d["batch_steps"]["realizations_per_step"] >= 1
    assert abs(d["ms_per_step"] - 1000.0 * per_step / d["value"]) < 1e-6 * d["ms_per_step"] + 1e-9
    assert d["batch_steps"]["plain_value"] > 0
    rf = d["roofline"]
    assert rf["bound"] in ("hbm", "tensor") and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert d["cpu_baseline"]["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert set(d["stage_ms"]) == {"noise", "front", "fill", "route", "trace", "border"}
