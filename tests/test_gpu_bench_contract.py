"""bench.py keeps its JSON-line contract on a small run of each workload.

One JSON line on stdout with the metric, the whole-job value, the timing
fields, the roofline of the dominant kernel (algorithmic bytes per launch
over its event-timed duration, against the measured copy peak), the
end-to-end leg with its host-link bytes, the kernel launches counted inside
the timed region and the clocks sampled during it.
"""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def _line(*args):
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True,
                         text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(x) for x in res.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, res.stdout[-2000:]
    return lines[0]


def _common(b, steps, warmup):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "roofline", "e2e", "gpu_launches", "clocks"):
        assert k in b, k
    assert b["n_gpus"] == 1 and b["steps"] == steps and b["warmup"] == warmup
    assert b["value"] > 0 and b["ms_per_step"] > 0 and b["higher_is_better"] is True
    assert "workload" in b["config"]
    r = b["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] > 0
    assert 0 < r["frac"] < 1.5 and abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-3
    e = b["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert "sm_mhz" in b["clocks"] and "reasons" in b["clocks"]


def test_suite_line():
    b = _line("--steps", "3", "--warmup", "3", "--problems", "4", "--no-cpu")
    _common(b, 3, 3)
    assert b["unit"] == "GB/s" and b["gpu_launches"] == 3 * 4
    assert 0 < b["geomean_frac_of_copy"] < 1.5


def test_grouped_line():
    b = _line("--workload", "grouped", "--problems", "200", "--steps", "3", "--warmup", "3",
              "--no-cpu", "--no-tune")
    _common(b, 3, 3)
    assert b["unit"] == "transposes/s"
    assert b["speedup_vs_loop"] > 1 and b["gpu_launches"] == 3 * b["config"]["buckets"]
