"""Evaluate the learned plan selector on the device.

For held-out problems of the selector's distribution (a seed not used in
training): planning latency of librettPlan with the learned model and with
the analytic model (plan cache off), of librettPlanMeasure (which times
every candidate), and of a repeated librettPlan served by the plan cache;
and the measured execute time of the learned and the analytic choice.

With --all-candidates every candidate of the default set is timed too, so
each selector's regret against the measured best is known per problem; with
--librett-choice (oracle/ref_bench/run_ref.py --choice output for the same
problems and seed) LibreTT's analytic GpuModel pick (its librettPlan) and its
librettPlanMeasure pick are joined per problem.

Usage (on a GPU):
    python -m librett_gb300.learn.evaluate --problems 200 --seed 424242 --out eval.json \
        [--all-candidates] [--librett-choice reference_choice.json]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
import time

import numpy as np

import librett_gb300 as L
from librett_gb300 import _lib

from .data import problems


def _time_exec(plan, din, dout, stream, ev):
    nbytes = int(np.prod(plan.dim)) * plan.sizeofType
    est = 2.0 * nbytes / 5e12 + 4e-6
    reps = int(min(64, max(1, np.ceil(200e-6 / est))))
    plan.execute(din, dout)
    ts = []
    for _ in range(3):
        ev[0].record(stream)
        for _ in range(reps):
            plan.execute(din, dout)
        ev[1].record(stream)
        ev[1].synchronize()
        ts.append(ev[0].elapsed_time(ev[1]) / reps / 1e3)
    return float(np.median(ts))


def evaluate(probs, all_candidates=False):
    import torch

    lib = _lib.load()
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    maxb = max(int(np.prod(d)) * es for d, _, es in probs)
    a = torch.empty(maxb, dtype=torch.uint8, device="cuda")
    b = torch.empty(maxb, dtype=torch.uint8, device="cuda")
    a.random_(0, 256)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    rows = []
    prev = lib.librett_c_set_plan_selector(0)
    prev_cache = lib.librett_c_set_plan_cache(0)  # every latency below is a full planning
    try:
        for dims, perm, es in probs:
            r = {"dims": dims, "perm": perm, "es": es}
            dims_c, perm_c = _lib.int_array(dims), _lib.int_array(perm)
            for mode, name in ((1, "analytic"), (2, "learned")):
                lib.librett_c_set_plan_selector(mode)
                torch.cuda.synchronize()
                # the C-ABI call alone (what a C/C++ caller pays)
                h = ctypes.c_uint(0)
                t0 = time.perf_counter()
                rc = lib.librett_c_plan(ctypes.byref(h), len(dims), dims_c, perm_c, es, sptr)
                r[f"plan_ms_{name}"] = (time.perf_counter() - t0) * 1e3
                assert rc == 0
                lib.librett_c_destroy(h.value)
                plan = L.Plan(dims, perm, es, stream)
                info = plan.info()
                r[f"selected_by_{name}"] = info["selected_by"]
                r[f"candidate_{name}"] = info["candidate"]
                r[f"exec_ms_{name}"] = _time_exec(plan, a.data_ptr(), b.data_ptr(), stream, ev) * 1e3
                plan.destroy()
            torch.cuda.synchronize()
            h = ctypes.c_uint(0)
            t0 = time.perf_counter()
            rc = lib.librett_c_plan_measure(ctypes.byref(h), len(dims), dims_c, perm_c, es, sptr,
                                            a.data_ptr(), b.data_ptr())
            r["plan_ms_measure"] = (time.perf_counter() - t0) * 1e3
            assert rc == 0
            lib.librett_c_destroy(h.value)
            plan = L.Plan(dims, perm, es, stream, measure=(a.data_ptr(), b.data_ptr()))
            r["exec_ms_measure"] = _time_exec(plan, a.data_ptr(), b.data_ptr(), stream, ev) * 1e3
            plan.destroy()
            if all_candidates:
                lib.librett_c_set_plan_selector(0)
                times = []
                for c in range(info["num_candidates"]):
                    plan = L.Plan(dims, perm, es, stream, candidate=c)
                    times.append(_time_exec(plan, a.data_ptr(), b.data_ptr(), stream, ev) * 1e3)
                    plan.destroy()
                r["exec_ms_candidates"] = times
                r["exec_ms_best"] = min(times + [r["exec_ms_learned"], r["exec_ms_analytic"],
                                                 r["exec_ms_measure"]])
            # a repeated shape with the plan cache on (the second call hits)
            lib.librett_c_set_plan_selector(0)
            lib.librett_c_set_plan_cache(16)
            for k in range(2):
                h = ctypes.c_uint(0)
                t0 = time.perf_counter()
                rc = lib.librett_c_plan(ctypes.byref(h), len(dims), dims_c, perm_c, es, sptr)
                r["plan_ms_cached"] = (time.perf_counter() - t0) * 1e3
                assert rc == 0
                lib.librett_c_destroy(h.value)
            lib.librett_c_set_plan_cache(0)
            rows.append(r)
    finally:
        lib.librett_c_set_plan_selector(prev)
        lib.librett_c_set_plan_cache(prev_cache)
    g = lambda x: float(np.exp(np.mean(np.log(x))))  # noqa: E731
    summary = {
        "problems": len(rows),
        "plan_ms_median": {k: float(np.median([r[f"plan_ms_{k}"] for r in rows]))
                           for k in ("learned", "analytic", "measure", "cached")},
        "learned_used": int(sum(r["selected_by_learned"] == 1 for r in rows)),
        "exec_time_ratio_learned_over_analytic_geomean":
            g([r["exec_ms_learned"] / r["exec_ms_analytic"] for r in rows]),
        "exec_time_ratio_learned_over_measure_geomean":
            g([r["exec_ms_learned"] / r["exec_ms_measure"] for r in rows]),
    }
    summary["plan_latency_measure_over_learned"] = (summary["plan_ms_median"]["measure"] /
                                                    summary["plan_ms_median"]["learned"])
    # by problem size
    buckets = {}
    for lo, hi in ((16, 20), (20, 24), (24, 29)):
        sel = [r for r in rows if lo <= np.log2(np.prod(r["dims"]) * r["es"]) < hi]
        if sel:
            buckets[f"2^{lo}..2^{hi} bytes"] = {
                "problems": len(sel),
                "learned_ms": float(np.median([r["plan_ms_learned"] for r in sel])),
                "measure_ms": float(np.median([r["plan_ms_measure"] for r in sel]))}
    summary["by_size"] = buckets
    if all_candidates:
        summary["regret_vs_best"] = {
            k: _regret([r[f"exec_ms_{k}"] / r["exec_ms_best"] for r in rows])
            for k in ("learned", "analytic", "measure")}
    return summary, rows


def _regret(ratios):
    """Geomean and p90 of t(pick) / t(best) - 1."""
    ratios = np.asarray(ratios, dtype=np.float64)
    return {"geomean": float(np.exp(np.mean(np.log(ratios)))) - 1,
            "p90": float(np.percentile(ratios, 90)) - 1,
            "exact_best": int(np.sum(ratios <= 1 + 1e-9))}


def join_librett(summary, rows, choice):
    """Adds LibreTT's per-problem picks (its librettPlan = the GpuModel
    choice, and its librettPlanMeasure choice) to the rows and the regret
    table: GpuModel's regret against LibreTT's own measured choice, and both
    LibreTT picks against the engine's measured best."""
    plan, meas = choice["plan"], choice["measure"]
    assert len(plan) == len(rows) == len(meas)
    for r, p, m in zip(rows, plan, meas):
        assert p["dims"] == r["dims"] and p["perm"] == r["perm"] and p["es"] == r["es"]
        r["librett_exec_ms_plan"] = p["ms"]
        r["librett_exec_ms_measure"] = m["ms"]
        r["librett_plan_ms"] = p["plan_ms"]
        r["librett_plan_measure_ms"] = m["plan_ms"]
    summary["librett"] = {
        "gpumodel_regret_vs_librett_measure": _regret(
            [max(1.0, r["librett_exec_ms_plan"] / r["librett_exec_ms_measure"]) for r in rows]),
        "plan_ms_median": {"librettPlan": float(np.median([r["librett_plan_ms"] for r in rows])),
                           "librettPlanMeasure": float(np.median(
                               [r["librett_plan_measure_ms"] for r in rows]))},
    }
    if "exec_ms_best" in rows[0]:
        summary["librett"]["gpumodel_vs_engine_best"] = _regret(
            [r["librett_exec_ms_plan"] / r["exec_ms_best"] for r in rows])
        summary["librett"]["librett_measure_vs_engine_best"] = _regret(
            [r["librett_exec_ms_measure"] / r["exec_ms_best"] for r in rows])
    return summary


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--problems", type=int, default=200)
    ap.add_argument("--seed", type=int, default=424242)
    ap.add_argument("--out", default=None)
    ap.add_argument("--all-candidates", action="store_true",
                    help="time every candidate of every problem (regret against the best)")
    ap.add_argument("--librett-choice", default=None,
                    help="run_ref.py --choice output for the same problems: join LibreTT's picks")
    args = ap.parse_args(argv)
    import torch

    torch.cuda.set_device(0)
    summary, rows = evaluate(problems(args.problems, args.seed), args.all_candidates)
    if args.librett_choice:
        with open(args.librett_choice) as f:
            summary = join_librett(summary, rows, json.load(f))
    print(json.dumps(summary, indent=1))
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"summary": summary, "rows": rows}, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
