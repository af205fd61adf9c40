"""Build and run LibreTT's own CUDA build -- TEST INFRASTRUCTURE ONLY.

Compiles LibreTT's library sources, unmodified, from a source directory
together with ref_driver.cpp into oracle/_ref/ref_driver with nvcc for
sm_103a.  The source directory is --src, else the LIBRETT_REF_SRC
environment variable, else a staged copy in oracle/_ref/src (git-ignored;
`--stage` makes it, so that a machine without the LibreTT checkout -- the
GPU machine -- can compile the checker), else the checkout's src/ on the
development machine (DEFAULT_SRC).  Nothing from LibreTT is committed.
With --engine the same driver source is also compiled against this engine's
include/librett.h and linked with librett_gb300/librett.so
(oracle/_ref/engine_driver): the driver only calls the LibreTT API, so both
libraries are timed by identical code.
Then, for LibreTT (and for the engine with --engine):

  --golden : runs every case of tests/golden/golden.json through
             librettPlan + librettExecute and compares the sha256 of each
             output with the fixture (pins the fixtures to LibreTT itself);
  --bench  : times the small case, the two small-leading-dimension cases and
             the first --suite problems of the random-shape suite;
  --loop N : times the per-tensor librettExecute loop over N problems of the
             batched distribution (librett_gb300.workloads);
  --planning N : times librettPlan and librettPlanMeasure on N problems of
             the plan-selection distribution;
  --random : runs the benchmark configurations (C1, C3a, C3b, the first 40
             suite problems, the first 20 batched problems) on the seeded
             random inputs of oracle/vectors.py and digests every output;
             with --write-fixture, LibreTT's digests become
             tests/golden/librett_random.json;
  --choice N : executes LibreTT's librettPlan pick and its
             librettPlanMeasure pick of N problems of the plan-selection
             distribution (10 timed launches each): the per-problem record
             of the analytic GpuModel's choice.

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
import shutil
import statistics
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF = ROOT / "oracle" / "_ref"
STAGED_SRC = REF / "src"
DEFAULT_SRC = Path("/root/reference/src")  # the LibreTT checkout on the development machine
DRIVER = REF / "ref_driver"
ENGINE_DRIVER = REF / "engine_driver"
LIB_SOURCES = ["librett.cpp", "plan.cpp", "kernel.cpp", "GpuModel.cpp", "GpuModelKernel.cpp",
               "GpuUtils.cpp", "Timer.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def source_dir(src=None):
    """LibreTT's src/ to compile from, or None when none is present."""
    for cand in (src, os.environ.get("LIBRETT_REF_SRC"), STAGED_SRC, DEFAULT_SRC):
        if cand and (Path(cand) / "librett.h").is_file():
            return Path(cand)
    return None


def stage(src: Path) -> Path:
    """Copies LibreTT's library sources and headers into the git-ignored
    oracle/_ref/src, which travels with the working tree to the GPU machine."""
    STAGED_SRC.mkdir(parents=True, exist_ok=True)
    for f in Path(src).iterdir():
        if f.suffix in (".cpp", ".h", ".hpp") and f.is_file():
            shutil.copy2(f, STAGED_SRC / f.name)
    return STAGED_SRC


def build(src: Path) -> Path:
    """Compiles LibreTT's sources (in parallel) and the driver, links
    oracle/_ref/ref_driver."""
    src = Path(src)
    obj = REF / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    units = [src / f for f in LIB_SOURCES] + [HERE / "ref_driver.cpp"]

    def compile_one(f):
        o = obj / (f.name + ".o")
        subprocess.run([nvcc, "-O3", "-std=c++17", "-DLIBRETT_USES_CUDA", *ARCH, "-w",
                        f"-I{src}", "-x", "cu", "-c", str(f), "-o", str(o)], check=True)
        return o

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    subprocess.run([nvcc, *ARCH, *map(str, objs), "-o", str(DRIVER)], check=True)
    return DRIVER


def build_engine() -> Path:
    """The same driver linked against this engine (the drop-in path)."""
    REF.mkdir(parents=True, exist_ok=True)
    sys.path.insert(0, str(ROOT))
    from librett_gb300.build import build as build_lib

    lib = build_lib()
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, "-O3", "-std=c++17", *ARCH, f"-I{ROOT / 'include'}", "-x", "cu",
           str(HERE / "ref_driver.cpp"), "-o", str(ENGINE_DRIVER), f"-L{lib.parent}", "-l:librett.so",
           "-Xlinker", f"-rpath={lib.parent}"]
    subprocess.run(cmd, check=True)
    return ENGINE_DRIVER


def write_cases(path: Path, cases):
    """One line per case; kind "value"/"words"/"none", or an int key for
    seeded random words (kind 3)."""
    kinds = {"value": 0, "words": 1, "none": 2}
    with open(path, "w") as f:
        for dims, perm, es, kind in cases:
            tail = [3, int(kind)] if isinstance(kind, int) else [kinds[kind]]
            f.write(" ".join(map(str, [len(dims), *dims, *perm, es, *tail])) + "\n")


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


FIXTURE = ROOT / "tests" / "golden" / "librett_random.json"
RANDOM_KEY0 = 0x6C69627265747400  # first key; case n uses RANDOM_KEY0 + n


def random_cases():
    """(name, dims, perm, es) of the benchmark configurations pinned by
    LibreTT's outputs on seeded random inputs."""
    sys.path.insert(0, str(ROOT))
    import bench as B
    from librett_gb300.workloads import grouped_problems

    cases = [("c1", *B.workload_problems("c1", 1)[0]),
             ("c3a", *B.workload_problems("c3a", 1)[0]),
             ("c3b", *B.workload_problems("c3b", 1)[0])]
    cases += [(f"suite{i}", *p) for i, p in enumerate(B.suite_problems(200)[:40])]
    cases += [(f"grouped{i}", *p) for i, p in enumerate(grouped_problems(20))]
    return cases


def run_random(out: Path, driver: Path, prefix: str) -> list:
    """Runs every random case through the driver and digests each output
    as it streams back (oracle/vectors.py tree digest)."""
    sys.path.insert(0, str(ROOT))
    from oracle.vectors import StreamDigest

    cases = random_cases()
    cf = out / "random_cases.txt"
    write_cases(cf, [(d, p, es, RANDOM_KEY0 + n) for n, (_, d, p, es) in enumerate(cases)])
    proc = subprocess.Popen([str(driver), "random", str(cf)], stdout=subprocess.PIPE)
    rows = []
    for n, (name, dims, perm, es) in enumerate(cases):
        head = proc.stdout.read(8)
        if len(head) != 8:
            break
        nbytes = int.from_bytes(head, "little")
        sd = StreamDigest()
        left = nbytes
        while left:
            piece = proc.stdout.read(min(left, 16 << 20))
            if not piece:
                raise RuntimeError(f"{prefix}: output of case {name} cut short")
            sd.update(piece)
            left -= len(piece)
        rows.append({"name": name, "dims": dims, "perm": perm, "es": es,
                     "key": RANDOM_KEY0 + n, "bytes": nbytes, "digest": sd.hexdigest()})
    if proc.wait() != 0 or len(rows) != len(cases):
        raise RuntimeError(f"{prefix} driver failed in random mode after {len(rows)} cases")
    (out / f"{prefix}_random.json").write_text(json.dumps(rows, indent=1) + "\n")
    return rows


def write_fixture(rows: list, engine_rows=None, path: Path = FIXTURE) -> None:
    doc = {
        "what": "digests of LibreTT's own outputs on seeded random inputs at the benchmark "
                "configurations",
        "input": "oracle/vectors.py: little-endian words mix64(key + (i + 1) * 0x9E3779B97F4A7C15)",
        "digest": "oracle/vectors.py tree_digest: sha256 of the sha256 digests of 64 MiB chunks",
        "generated_by": "oracle/ref_bench/run_ref.py --random --write-fixture: LibreTT's src/, "
                        "unmodified, compiled for sm_103a; librettPlan + librettExecute on a GB300",
        "cases": rows,
    }
    if engine_rows is not None:
        doc["engine_matching_at_generation"] = sum(
            a["digest"] == b["digest"] for a, b in zip(rows, engine_rows))
    Path(path).write_text(json.dumps(doc, indent=1) + "\n")


def run_choice(out: Path, driver: Path, prefix: str, n: int, seed: int):
    """LibreTT's librettPlan (GpuModel) pick and librettPlanMeasure pick of
    n problems of the plan-selection distribution, each executed 10 times
    after 3 warm-up launches."""
    sys.path.insert(0, str(ROOT))
    from librett_gb300.learn.data import problems

    cases = [(d, p, es, "none") for d, p, es in problems(n, seed)]
    cf = out / "choice_cases.txt"
    write_cases(cf, cases)
    res = {}
    for measure in (0, 1):
        r = subprocess.run([str(driver), "bench", str(cf), "10", "3", str(measure)], check=True,
                           capture_output=True, text=True)
        res["measure" if measure else "plan"] = _json_lines(r.stdout)
    (out / f"{prefix}_choice.json").write_text(json.dumps(res) + "\n")
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
    ap.add_argument("--src", default=None,
                    help="LibreTT's src/ (default: LIBRETT_REF_SRC, the staged copy, or the "
                         "development machine's checkout)")
    ap.add_argument("--stage", action="store_true",
                    help="copy LibreTT's sources into the git-ignored oracle/_ref/src and exit")
    ap.add_argument("--random", action="store_true")
    ap.add_argument("--write-fixture", nargs="?", const=str(FIXTURE), default=None,
                    help="with --random: write LibreTT's digests to this file "
                         "(default tests/golden/librett_random.json)")
    ap.add_argument("--choice", type=int, default=0)
    ap.add_argument("--choice-seed", type=int, default=424242)
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
    src = source_dir(args.src)
    if args.stage:
        if src is None or src == STAGED_SRC:
            raise SystemExit("no LibreTT source directory to stage from")
        print(stage(src))
        return 0
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    drivers = []
    if not args.engine_only:
        if src is None:
            raise SystemExit("LibreTT's sources are not present (set LIBRETT_REF_SRC)")
        drivers.append((build(src), "reference"))
    if args.engine or args.engine_only:
        drivers.append((build_engine(), "engine"))
    random_rows = {}
    for driver, prefix in drivers:
        if args.random:
            random_rows[prefix] = run_random(out, driver, prefix)
            print(f"{prefix} random: {len(random_rows[prefix])} cases digested")
        if args.choice:
            run_choice(out, driver, prefix, args.choice, args.choice_seed)
            print(f"{prefix} choice: {args.choice} problems")
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
    if "reference" in random_rows and "engine" in random_rows:
        same = sum(a["digest"] == b["digest"]
                   for a, b in zip(random_rows["reference"], random_rows["engine"]))
        print(f"random: engine matches LibreTT on {same}/{len(random_rows['reference'])} cases")
    if args.random and args.write_fixture and "reference" in random_rows:
        write_fixture(random_rows["reference"], random_rows.get("engine"), args.write_fixture)
        print(f"wrote {args.write_fixture}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
