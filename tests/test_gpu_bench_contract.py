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
    b = _line("--steps", "3", "--warmup", "3", "--problems", "4", "--no-cpu", "--no-extras")
    _common(b, 3, 3)
    assert b["unit"] == "GB/s" and b["gpu_launches"] == 3 * 4
    assert 0 < b["geomean_frac_of_copy"] < 1.5
    assert b["verified"] == 4
    link = b["e2e"]["link_ceiling_same_run"]
    assert link["h2d_gbs"] > 0 and link["d2h_gbs"] > 0 and link["bidirectional_gbs"] > 0


def test_suite_line_with_the_other_configurations():
    """The default line also carries C1, C3a, C3b, the grouped batch,
    planning latency and plan-choice regret, each measured in the run (here
    on reduced counts)."""
    b = _line("--steps", "3", "--warmup", "3", "--problems", "2", "--no-cpu",
              "--grouped-problems", "300", "--planning-problems", "12",
              "--selection-problems", "6", "--extra-cpu-budget", "0.2")
    c = b["configs"]
    for name in ("c1", "c3a", "c3b"):
        assert c[name]["verified"] is True and c[name]["gbs"] > 0
        r = c[name]["roofline"]
        assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-3
        assert c[name]["cpu_baseline"]["value"] > 0
    g = c["grouped"]
    assert g["verified"] == g["members"] == 300 and g["speedup_vs_loop"] > 1
    assert c["planning"]["problems"] == 12 and c["planning"]["ratio"] > 1
    assert c["selection"]["problems"] == 6
    assert set(c["selection"]["regret_geomean"]) == {"learned", "analytic"}
    assert "reason" in c["librett_cuda"] or c["librett_cuda"]["c3a"]["gbs_plan"] > 0


def test_grouped_line():
    b = _line("--workload", "grouped", "--problems", "200", "--steps", "3", "--warmup", "3",
              "--no-cpu", "--no-tune")
    _common(b, 3, 3)
    assert b["unit"] == "transposes/s"
    assert b["speedup_vs_loop"] > 1 and b["gpu_launches"] == 3 * b["config"]["buckets"]
