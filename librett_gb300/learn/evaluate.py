"""Evaluate the learned plan selector on the device.

For held-out problems of the selector's distribution (a seed not used in
training): planning latency of librettPlan with the learned model and with
the analytic model (plan cache off), of librettPlanMeasure (which times
every candidate), and of a repeated librettPlan served by the plan cache;
and the measured execute time of the learned and the analytic choice.

Usage (on a GPU):
    python -m librett_gb300.learn.evaluate --problems 200 --seed 424242 --out eval.json
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


def evaluate(probs):
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
    return summary, rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--problems", type=int, default=200)
    ap.add_argument("--seed", type=int, default=424242)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    import torch

    torch.cuda.set_device(0)
    summary, rows = evaluate(problems(args.problems, args.seed))
    print(json.dumps(summary, indent=1))
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"summary": summary, "rows": rows}, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
