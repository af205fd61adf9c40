"""Benchmark of the transpose engine on one GB300 (or N replicas).

Default workload: the random-shape suite (200 problems from a fixed seed;
rank uniform in 2..7; dims drawn log-uniformly with product within 5% of
2^27 elements; uniformly random permutation; float64 holding random 64-bit
patterns, 1 GiB in + 1 GiB out per problem).  One step = one execute of
every problem's plan, plans created before timing.  Inputs (1 GiB) are far
larger than L2 (126 MB), so no L2 flush is needed between launches.

Metric (LibreTT src/Timer.cpp:151): effective GB/s = 2 * vol * sizeof / t,
summed over the problems of a step.  Reported with the HBM roofline of the
dominant kernel, a CPU baseline (the oracle's multithreaded host gather
loop on a bounded sample), an end-to-end number through the public C-ABI
with pinned host buffers, the SM clocks seen during the timed region, and
the number of this library's kernel launches in the timed region.

--impl reference times the CPU implementation of the path (the oracle's
host gather loop, all host threads) on the same workload; LibreTT has no
CPU transpose of its own.

Multi-GPU: the path does not shard (one transpose is one launch); N > 1
runs N independent replicas under torchrun and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SUITE_SEED = 20270127
SUITE_LOG2_VOL = 27


def suite_problems(n=200, seed=SUITE_SEED):
    """Random-shape suite: rank U{2..7}; weights w_r ~ U(0,1) scaled so that
    sum log2 d = 27; d >= 2; product fixed to within +-5% of 2^27; random
    permutation (identities kept; they fuse to a plain copy)."""
    rng = np.random.Generator(np.random.MT19937(seed))
    target = 2 ** SUITE_LOG2_VOL
    out = []
    for _ in range(n):
        rank = int(rng.integers(2, 8))
        w = rng.uniform(0.0, 1.0, rank)
        logd = w / w.sum() * SUITE_LOG2_VOL
        dims = [max(2, int(round(2.0 ** x))) for x in logd]
        for _ in range(64):
            vol = int(np.prod(dims))
            if abs(vol - target) <= 0.05 * target:
                break
            i = int(np.argmax(dims))
            dims[i] = max(2, int(round(dims[i] * target / vol)))
        perm = [int(x) for x in rng.permutation(rank)]
        out.append((dims, perm, 8))
    return out


WORKLOADS = {
    "suite": "random-shape suite, 200 problems, rank 2..7, ~2^27 float64 elements each",
    "c3a": "complex128 dims (4,6,8192,5,256) perm (3,0,4,2,1)",
    "c3b": "float32 dims (2,3,4,5,65536,16) perm (5,3,1,4,0,2)",
    "c1": "float32 dims (64,48,32) perm (2,0,1)",
    "custom": "one problem given by --dims/--perm/--es",
}


def workload_problems(name, nproblems, custom=None):
    if name == "custom":
        return [custom]
    if name == "suite":
        return suite_problems(nproblems)
    if name == "c3a":
        return [([4, 6, 8192, 5, 256], [3, 0, 4, 2, 1], 16)]
    if name == "c3b":
        return [([2, 3, 4, 5, 65536, 16], [5, 3, 1, 4, 0, 2], 4)]
    if name == "c1":
        return [([64, 48, 32], [2, 0, 1], 4)]
    raise ValueError(name)


def problem_bytes(p):
    dims, _, es = p
    return int(np.prod(dims)) * es


def load_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        loaded = [x for x in sm if x > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup(n_gpus):
    import torch
    import torch.distributed as dist

    if n_gpus > 1 or int(os.environ.get("WORLD_SIZE", "1")) > 1:
        rank = int(os.environ.get("RANK", "0"))
        local = int(os.environ.get("LOCAL_RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        torch.cuda.set_device(local) if torch.cuda.is_available() else None
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend, rank=rank, world_size=world)
        return rank, local, world
    return 0, 0, 1


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU legs (oracle host loop)
# ---------------------------------------------------------------------------

def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_gather_time(problems, budget_s, threads, rng_seed=1):
    """Time the oracle's host gather over problems until budget_s is spent."""
    from oracle import oracle as O

    maxb = max(problem_bytes(p) for p in problems)
    src = np.random.default_rng(rng_seed).integers(0, 256, maxb, dtype=np.uint8)
    dst = np.empty(maxb, dtype=np.uint8)
    dst[:] = 0  # fault pages in before timing
    done, t_total, bytes_total = 0, 0.0, 0
    for p in problems:
        dims, perm, es = p
        nb = problem_bytes(p)
        t0 = time.perf_counter()
        O.transpose_c(src[:nb], dims, perm, es, threads, out=dst[:nb])
        t_total += time.perf_counter() - t0
        bytes_total += 2 * nb
        done += 1
        if t_total >= budget_s:
            break
    return bytes_total / t_total / 1e9, done, t_total


def run_reference(args):
    rank, _, world = dist_setup(args.gpus)
    problems = workload_problems(args.workload, args.problems, args.custom)
    if rank != 0:
        return 0
    threads = host_threads()
    from oracle import oracle as O  # noqa: F401  (built before timing)
    O.build_oracle()
    # warm-up steps: one problem each
    for i in range(args.warmup):
        cpu_gather_time([problems[i % len(problems)]], 0.0, threads)
    gbs_t, bytes_t = 0.0, 0
    t_all = 0.0
    for i in range(args.steps):
        p = problems[(args.warmup + i) % len(problems)]
        gbs, _, t = cpu_gather_time([p], 0.0, threads)
        t_all += t
        bytes_t += 2 * problem_bytes(p)
    value = bytes_t / t_all / 1e9
    line = {
        "impl": "reference", "metric": "effective GB/s (2*bytes/time)", "value": round(value, 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_all / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.workload == "suite" else "bits",
        "data": "synthetic random 64-bit patterns",
        "config": {"workload": WORKLOADS[args.workload], "problems_per_step": 1,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"one suite problem per step, {args.steps} steps"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def traffic_from_profiles(workload):
    f = ROOT / "profiles" / f"traffic_{workload}.json"
    if not f.exists():
        return None
    try:
        return json.loads(f.read_text())
    except json.JSONDecodeError:
        return None


def run_engine(args):
    import torch

    import librett_gb300 as L

    rank, local, world = dist_setup(args.gpus)
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    problems = workload_problems(args.workload, args.problems, args.custom)
    stream = torch.cuda.current_stream(dev)
    maxb = max(problem_bytes(p) for p in problems)
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    inp = torch.randint(-(2 ** 62), 2 ** 62, ((maxb + 7) // 8,), dtype=torch.int64, device=dev,
                        generator=g).view(torch.uint8)[:maxb]
    out = torch.empty(maxb, dtype=torch.uint8, device=dev)
    plans = [L.Plan(d, p, es, stream, candidate=args.candidate) for d, p, es in problems]
    infos = [pl.info() for pl in plans]
    ip, op = inp.data_ptr(), out.data_ptr()
    step_bytes = sum(2 * problem_bytes(p) for p in problems)

    def step(events=None):
        for k, pl in enumerate(plans):
            if events is not None:
                events[k][0].record(stream)
            pl.execute(ip, op)
            if events is not None:
                events[k][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in plans] for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize(dev)
    launches0 = L.launch_count()
    t0.record(stream)
    for s in range(args.steps):
        step(ev[s])
    t1.record(stream)
    torch.cuda.synchronize(dev)
    launches = L.launch_count() - launches0
    barrier(world)
    clk = clocks.stop()
    ms = t0.elapsed_time(t1)
    ms_max = max_over_ranks(ms, world)
    value = world * step_bytes * args.steps / (ms_max / 1e3) / 1e9

    # per-kernel breakdown from the per-launch events
    per_kernel = {}
    per_problem_ms = []
    for k, info in enumerate(infos):
        name = L.METHOD_NAMES[info["method"]]
        kname = {"Trivial": "copyKernel", "TiledCopy": "rowCopyKernel"}.get(name, "tileKernel")
        ts = [ev[s][k][0].elapsed_time(ev[s][k][1]) for s in range(args.steps)]
        t = statistics.median(ts)
        per_problem_ms.append(t)
        pk = per_kernel.setdefault(kname, {"launches": 0, "ms": 0.0, "bytes": 0})
        pk["launches"] += args.steps
        pk["ms"] += sum(ts)
        pk["bytes"] += 2 * problem_bytes(problems[k]) * args.steps
    if args.per_problem:
        with open(args.per_problem, "w") as fpp:
            for (dims, perm, es), t, info in zip(problems, per_problem_ms, infos):
                fpp.write(json.dumps({"dims": dims, "perm": perm, "es": es, "ms": t,
                                      "gbs": 2 * problem_bytes((dims, perm, es)) / (t / 1e3) / 1e9,
                                      "method": info["method"], "pipeline": info["pipeline"],
                                      "tile": info["tile_extent"]}) + "\n")
    dom = max(per_kernel, key=lambda n: per_kernel[n]["ms"])
    d = per_kernel[dom]
    peak, peak_kind = load_peaks()
    achieved = d["bytes"] / d["launches"] / (d["ms"] / d["launches"] / 1e3) / 1e9
    prof = traffic_from_profiles(args.workload)
    traffic = None
    if prof and prof.get("kernel") == dom:
        traffic = prof.get("dram_bytes_per_launch")
    geo = float(np.exp(np.mean([np.log(2 * problem_bytes(p) / (t / 1e3) / 1e9)
                                for p, t in zip(problems, per_problem_ms)])))

    # end to end through the public API: pinned host in -> device -> host out
    e2e = None
    if not args.no_e2e:
        hin = torch.empty(maxb, dtype=torch.uint8, pin_memory=True)
        hin.copy_(inp.cpu())
        hout = torch.empty(maxb, dtype=torch.uint8, pin_memory=True)

        def e2e_step():
            for (dims, perm, es), pl in zip(problems, plans):
                nb = problem_bytes((dims, perm, es))
                inp[:nb].copy_(hin[:nb], non_blocking=True)
                pl.execute(ip, op)
                hout[:nb].copy_(out[:nb], non_blocking=True)

        e2e_step()
        torch.cuda.synchronize(dev)
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e2e_step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ems = max_over_ranks(e0.elapsed_time(e1), world)
        e2e = {"value": round(world * step_bytes / (ems / 1e3) / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": step_bytes // 2, "d2h_bytes_per_step": step_bytes // 2,
               "ms_per_step": round(ems, 3)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        gbs, n, t = cpu_gather_time(problems, args.cpu_budget, host_threads())
        cpu = {"value": round(gbs, 3), "unit": "GB/s", "cores": host_threads(), "kind": "port",
               "sample": f"first {n} problem(s) of the workload, {t:.1f} s of host gather"}

    if rank != 0:
        return 0
    methods = {}
    for info in infos:
        nm = L.METHOD_NAMES[info["method"]]
        methods[nm] = methods.get(nm, 0) + 1
    line = {
        "metric": "effective GB/s (2*bytes/time)",
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {4: "u32", 8: "u64", 16: "u128"}[problems[0][2]],
        "data": "synthetic random 64-bit patterns, fixed seeds",
        "config": {"workload": WORKLOADS[args.workload] if args.workload != "custom"
                   else f"dims {problems[0][0]} perm {problems[0][1]} {problems[0][2]}-byte",
                   "problems": len(problems), "candidate": args.candidate,
                   "suite_seed": SUITE_SEED if args.workload == "suite" else None,
                   "bytes_per_step": step_bytes, "l2": "inputs larger than L2, no flush",
                   "parallelism": f"replicas x{world}", "methods": methods},
        "geomean_gbs": round(geo, 3),
        "geomean_frac_of_copy": round(geo / peak, 4),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 3),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind,
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": d["bytes"] // d["launches"]},
        "per_kernel": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                           "gbs": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1)}
                       for k, v in per_kernel.items()},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    for pl in plans:
        pl.destroy()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="suite")
    ap.add_argument("--problems", type=int, default=200)
    ap.add_argument("--cpu-budget", type=float, default=12.0,
                    help="seconds of host gather for the cpu_baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--dims", type=str, default=None, help="custom problem: comma-separated dims")
    ap.add_argument("--perm", type=str, default=None, help="custom problem: permutation")
    ap.add_argument("--es", type=int, default=8, help="custom problem: element bytes")
    ap.add_argument("--per-problem", type=str, default=None,
                    help="write one JSON line per problem (median launch time) to this file")
    ap.add_argument("--candidate", type=int, default=None,
                    help="plan every problem with this planner candidate (default: heuristic)")
    args = ap.parse_args(argv)
    args.custom = None
    if args.dims:
        args.workload = "custom"
        args.custom = ([int(x) for x in args.dims.split(",")],
                       [int(x) for x in args.perm.split(",")], args.es)
    if args.impl == "reference":
        return run_reference(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())
