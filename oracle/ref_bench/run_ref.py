"""Build and run LibreTT's own CUDA build -- TEST INFRASTRUCTURE ONLY.

Compiles LibreTT's library sources, unmodified, from a source directory
(default: the LibreTT checkout's src/) together with ref_driver.cpp into
oracle/_ref/ref_driver with nvcc for sm_103a.  With --engine the same
driver source is also compiled against this engine's include/librett.h and
linked with librett_gb300/librett.so (oracle/_ref/engine_driver): the driver
only calls the LibreTT API, so both libraries are timed by identical code.
Then, for LibreTT (and for the engine with --engine):

  --golden : runs every case of tests/golden/golden.json through
             librettPlan + librettExecute and compares the sha256 of each
             output with the fixture (pins the fixtures to LibreTT itself);
  --bench  : times the small case, the two small-leading-dimension cases and
             the first --suite problems of the random-shape suite;
  --loop N : times the per-tensor librettExecute loop over N problems of the
             batched distribution (librett_gb300.workloads);
  --planning N : times librettPlan and librettPlanMeasure on N problems of
             the plan-selection distribution.

Usage: python oracle/ref_bench/run_ref.py --src <LibreTT src dir> --out <dir>
       [--engine] [--golden] [--bench] [--suite N] [--measure] [--loop N]
       [--planning N]
Writes JSON results under --out (files prefixed reference_ / engine_).
Nothing here is used by the engine.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = ROOT / "oracle" / "_ref"
DRIVER = REF / "ref_driver"
ENGINE_DRIVER = REF / "engine_driver"
LIB_SOURCES = ["librett.cpp", "plan.cpp", "kernel.cpp", "GpuModel.cpp", "GpuModelKernel.cpp",
               "GpuUtils.cpp", "Timer.cpp"]


def build(src: Path) -> Path:
    REF.mkdir(parents=True, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, "-O3", "-std=c++17", "-DLIBRETT_USES_CUDA", "-gencode",
           "arch=compute_103a,code=sm_103a", "-w", f"-I{src}", "-x", "cu",
           *[str(src / f) for f in LIB_SOURCES], str(HERE / "ref_driver.cpp"), "-o", str(DRIVER)]
    subprocess.run(cmd, check=True)
    return DRIVER


def build_engine() -> Path:
    """The same driver linked against this engine (the drop-in path)."""
    REF.mkdir(parents=True, exist_ok=True)
    sys.path.insert(0, str(ROOT))
    from librett_gb300.build import build as build_lib

    lib = build_lib()
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, "-O3", "-std=c++17", f"-I{ROOT / 'include'}", str(HERE / "ref_driver.cpp"),
           "-o", str(ENGINE_DRIVER), f"-L{lib.parent}", "-l:librett.so",
           "-Xlinker", f"-rpath={lib.parent}"]
    subprocess.run(cmd, check=True)
    return ENGINE_DRIVER


def write_cases(path: Path, cases):
    kinds = {"value": 0, "words": 1, "none": 2}
    with open(path, "w") as f:
        for dims, perm, es, kind in cases:
            f.write(" ".join(map(str, [len(dims), *dims, *perm, es, kinds[kind]])) + "\n")


def _json_lines(text):
    return [json.loads(x) for x in text.splitlines() if x.startswith("{")]


def run_golden(out: Path, driver: Path, prefix: str) -> dict:
    rows = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())
    cases = [(r["dims"], r["perm"], r["es"], r["input"]) for r in rows]
    cf = out / "golden_cases.txt"
    write_cases(cf, cases)
    od = out / f"{prefix}_golden_bin"
    od.mkdir(parents=True, exist_ok=True)
    subprocess.run([str(driver), "golden", str(cf), str(od)], check=True)
    result = []
    for n, r in enumerate(rows):
        data = (od / f"out_{n}.bin").read_bytes()
        h = hashlib.sha256(data).hexdigest()
        result.append({"dims": r["dims"], "perm": r["perm"], "es": r["es"], "input": r["input"],
                       "match": h == r["sha256"], "sha256": h})
        (od / f"out_{n}.bin").unlink()
    od.rmdir()
    summary = {"cases": len(result), "matching": sum(x["match"] for x in result),
               "rows": result}
    (out / f"{prefix}_golden.json").write_text(json.dumps(summary, indent=1) + "\n")
    return summary


def run_bench(out: Path, driver: Path, prefix: str, nsuite: int, measure: bool,
              steps: int = 10, warmup: int = 3):
    sys.path.insert(0, str(ROOT))
    import bench as B

    cases = [(d, p, es, "none") for d, p, es in
             (B.workload_problems("c1", 1) + B.workload_problems("c3a", 1) +
              B.workload_problems("c3b", 1) + B.suite_problems(200)[:nsuite])]
    cf = out / "bench_cases.txt"
    write_cases(cf, cases)
    res = subprocess.run([str(driver), "bench", str(cf), str(steps), str(warmup),
                          "1" if measure else "0"], check=True, capture_output=True, text=True)
    lines = _json_lines(res.stdout)
    name = f"{prefix}_bench_measure.jsonl" if measure else f"{prefix}_bench.jsonl"
    (out / name).write_text("".join(json.dumps(x) + "\n" for x in lines))
    return lines


def run_planning(out: Path, driver: Path, prefix: str, n: int, seed: int):
    """librettPlan and librettPlanMeasure latency on n problems of the
    plan-selection distribution (librett_gb300.learn.data.problems)."""
    sys.path.insert(0, str(ROOT))
    from librett_gb300.learn.data import problems

    cases = [(d, p, es, "none") for d, p, es in problems(n, seed)]
    cf = out / "planning_cases.txt"
    write_cases(cf, cases)
    res = {}
    env = dict(os.environ, LIBRETT_PLAN_CACHE="0")  # every call plans in full
    for measure in (0, 1):
        r = subprocess.run([str(driver), "bench", str(cf), "1", "0", str(measure)], check=True,
                           capture_output=True, text=True, env=env)
        res["measure" if measure else "plan"] = _json_lines(r.stdout)
    (out / f"{prefix}_planning.json").write_text(json.dumps(res) + "\n")
    return res


def run_loop(out: Path, driver: Path, prefix: str, n: int, steps: int = 5, warmup: int = 3):
    sys.path.insert(0, str(ROOT))
    from librett_gb300.workloads import grouped_problems

    cases = [(d, p, es, "none") for d, p, es in grouped_problems(n)]
    cf = out / "loop_cases.txt"
    write_cases(cf, cases)
    res = subprocess.run([str(driver), "loop", str(cf), str(steps), str(warmup)], check=True,
                         capture_output=True, text=True)
    line = _json_lines(res.stdout)[0]
    (out / f"{prefix}_loop.json").write_text(json.dumps(line) + "\n")
    return line


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--src", default="/root/reference/src")
    ap.add_argument("--out", default=str(ROOT / "oracle" / "_ref" / "results"))
    ap.add_argument("--engine", action="store_true",
                    help="also run every mode with the same driver linked to this engine")
    ap.add_argument("--engine-only", action="store_true",
                    help="run the modes with the engine driver only (no LibreTT sources needed)")
    ap.add_argument("--golden", action="store_true")
    ap.add_argument("--bench", action="store_true")
    ap.add_argument("--measure", action="store_true", help="bench with librettPlanMeasure too")
    ap.add_argument("--suite", type=int, default=40)
    ap.add_argument("--planning", type=int, default=0,
                    help="time librettPlan and librettPlanMeasure on this many problems of the "
                         "plan-selection distribution")
    ap.add_argument("--planning-seed", type=int, default=424242)
    ap.add_argument("--loop", type=int, default=0,
                    help="time the per-tensor librettExecute loop over this many problems of the "
                         "batched distribution")
    args = ap.parse_args(argv)
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    drivers = []
    if not args.engine_only:
        drivers.append((build(Path(args.src)), "reference"))
    if args.engine or args.engine_only:
        drivers.append((build_engine(), "engine"))
    for driver, prefix in drivers:
        if args.golden:
            s = run_golden(out, driver, prefix)
            print(f"{prefix} golden: {s['matching']}/{s['cases']} outputs match the fixtures")
        if args.bench:
            lines = run_bench(out, driver, prefix, args.suite, False)
            print(f"{prefix} bench: {len(lines)} cases timed")
            if args.measure:
                lines = run_bench(out, driver, prefix, args.suite, True)
                print(f"{prefix} bench (plan measure): {len(lines)} cases timed")
        if args.planning:
            res = run_planning(out, driver, prefix, args.planning, args.planning_seed)
            print("%s planning: median plan_ms librettPlan %.3f, librettPlanMeasure %.3f" % (
                prefix, statistics.median(x["plan_ms"] for x in res["plan"]),
                statistics.median(x["plan_ms"] for x in res["measure"])))
        if args.loop:
            line = run_loop(out, driver, prefix, args.loop)
            print(f"{prefix} loop: " + json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
