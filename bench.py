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
    "grouped": "batched grouped execute: 10,000 transposes, rank 2..6, volume log-uniform "
               "2^10..2^22 elements, float32/float64 50/50, random permutations",
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
    if name == "grouped":
        from librett_gb300.workloads import grouped_problems
        return grouped_problems(nproblems)
    raise ValueError(name)


def problem_bytes(p):
    dims, _, es = p
    return int(np.prod(dims)) * es


def line_dtype(problems):
    return {4: "u32", 8: "u64", 16: "u128"}[problems[0][2]]


def workload_config(args, problems):
    """The `config` object, identical in the engine and reference lines of
    a workload."""
    return {"workload": WORKLOADS[args.workload] if args.workload != "custom"
            else f"dims {problems[0][0]} perm {problems[0][1]} {problems[0][2]}-byte",
            "problems": len(problems),
            "suite_seed": SUITE_SEED if args.workload == "suite" else None,
            "l2": "inputs larger than L2, no flush"
            if max(problem_bytes(p) for p in problems) > 256 << 20
            else "L2 flushed before every timed launch"}


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
        text = Path(self.path).read_text()
        os.unlink(self.path)
        after = False
        if not self._rows(text):
            # a region shorter than the sampling period: one reading right after it
            try:
                text = subprocess.run(
                    ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True,
                    timeout=30).stdout
                after = True
            except (OSError, subprocess.TimeoutExpired):
                return None
        rows = self._rows(text)
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
        out = {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax,
               "reasons": sorted(reasons), "samples": 0 if after else len(rows)}
        if after:
            out["note"] = "timed region shorter than the 100 ms sampling period: one reading after it"
        return out

    @staticmethod
    def _rows(text):
        rows = []
        for line in text.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        return rows


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


GROUP_SLICE = 100  # problems per reference-arm step of the grouped workload
E2E_CHUNKS = 8  # groups the grouped end-to-end prefix is cut into (4: 48.8k, 8: 51.8k, 16: 50.8k transposes/s)


def _reference_grouped(args, problems, threads):
    """Reference arm of the grouped workload: the oracle's host gather over
    consecutive slices of GROUP_SLICE problems, one slice per step."""
    t_all, n_all, b_all = 0.0, 0, 0
    for i in range(args.steps):
        lo = ((args.warmup + i) * GROUP_SLICE) % len(problems)
        sl = problems[lo:lo + GROUP_SLICE]
        _, n, t = cpu_gather_time(sl, float("inf"), threads)
        t_all += t
        n_all += n
        b_all += sum(2 * problem_bytes(p) for p in sl[:n])
    value = n_all / t_all
    line = {
        "impl": "reference", "metric": "transposes/s (grouped)", "value": round(value, 1),
        "unit": "transposes/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_all / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32/u64",
        "data": "synthetic random bit patterns",
        "config": {"workload": WORKLOADS["grouped"], "problems_per_step": GROUP_SLICE,
                   "parallelism": "host threads"},
        "gbs": round(b_all / t_all / 1e9, 3),
        "cpu_baseline": {"value": round(value, 1), "unit": "transposes/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{GROUP_SLICE} consecutive problems per step, {args.steps} steps"},
        "e2e": {"value": round(value, 1), "unit": "transposes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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
    if args.workload == "grouped":
        return _reference_grouped(args, problems, threads)
    # The K timed steps split the workload's problems into K consecutive
    # slices (all 200 suite problems at K = 20, the same sample as the engine
    # line's cpu_baseline); fewer problems than steps wrap around.
    per = max(1, -(-len(problems) // args.steps))
    bytes_t, t_all, timed = 0, 0.0, 0
    for i in range(args.steps):
        sl = [problems[(i * per + k) % len(problems)] for k in range(per)]
        _, n, t = cpu_gather_time(sl, float("inf"), threads)
        t_all += t
        bytes_t += sum(2 * problem_bytes(p) for p in sl[:n])
        timed += n
    value = bytes_t / t_all / 1e9
    line = {
        "impl": "reference", "metric": "effective GB/s (2*bytes/time)", "value": round(value, 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_all / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": line_dtype(problems),
        "data": "synthetic random 64-bit patterns, fixed seeds",
        "config": workload_config(args, problems),
        "parallelism": f"host threads x{threads}",
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{timed} problems in {args.steps} steps of {per} consecutive "
                                   f"problems (LibreTT has no CPU transpose: the oracle's host "
                                   f"gather restates its algorithm)"},
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


def copy_ceiling(inp, out, stream, nbytes, reps=10):
    """Copy ceilings measured in the same run (the role of LibreTT's
    bench memcpy mode, tests/librett_bench.cpp:879-955): cudaMemcpyAsync
    device to device, and this engine's own copy kernel (a rank-1 plan), each
    the best of `reps` event-timed copies of nbytes; GB/s = 2 * bytes / t."""
    import torch

    import librett_gb300 as L

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def best(fn):
        fn()
        ts = []
        for _ in range(reps):
            ev[0].record(stream)
            fn()
            ev[1].record(stream)
            ev[1].synchronize()
            ts.append(ev[0].elapsed_time(ev[1]))
        return 2 * nbytes / (min(ts) / 1e3) / 1e9

    memcpy = best(lambda: out[:nbytes].copy_(inp[:nbytes], non_blocking=True))
    with L.Plan([nbytes // 8], [0], 8, stream) as p:
        engine = best(lambda: p.execute(inp.data_ptr(), out.data_ptr()))
    return {"cuda_memcpy_d2d_gbs": round(memcpy, 1), "engine_copy_kernel_gbs": round(engine, 1),
            "bytes": nbytes, "how": f"best of {reps}, 2*bytes/time"}


def link_ceiling(hin, hout, dbuf, dbuf2, nbytes, reps=5):
    """Host-link ceilings for the end-to-end leg, measured in the same run:
    pinned host -> device alone, device -> pinned host alone, and both at
    once on two streams (copy engines); each the best of `reps`, GB/s of
    bytes moved (both directions counted for the concurrent pair)."""
    import torch

    dev = dbuf.device
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def best(fn, moved):
        fn()
        torch.cuda.synchronize(dev)
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize(dev)
            ev[0].record(s1)
            s2.wait_event(ev[0])
            fn()
            j = torch.cuda.Event()
            j.record(s2)
            s1.wait_event(j)
            ev[1].record(s1)
            ev[1].synchronize()
            ts.append(ev[0].elapsed_time(ev[1]))
        return moved / (min(ts) / 1e3) / 1e9

    def h2d():
        with torch.cuda.stream(s1):
            dbuf[:nbytes].copy_(hin[:nbytes], non_blocking=True)

    def d2h():
        with torch.cuda.stream(s2):
            hout[:nbytes].copy_(dbuf2[:nbytes], non_blocking=True)

    def both():
        h2d()
        d2h()

    return {"h2d_gbs": round(best(h2d, nbytes), 1), "d2h_gbs": round(best(d2h, nbytes), 1),
            "bidirectional_gbs": round(best(both, 2 * nbytes), 1), "bytes": nbytes,
            "how": f"pinned host memory, copy engines, best of {reps}"}


class DeviceData:
    """Random 64-bit patterns in a device buffer, and an L2 flush buffer."""

    def __init__(self, dev, nbytes, seed):
        import torch

        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.inp = torch.randint(-(2 ** 62), 2 ** 62, ((nbytes + 7) // 8,), dtype=torch.int64,
                                 device=dev, generator=g).view(torch.uint8)[:nbytes]
        self.out = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev) \
            if nbytes <= 256 << 20 else None


def time_launches(fn, stream, steps, warmup, flush=None):
    """Mean ms of fn() on `stream`: `steps` back-to-back launches between two
    events after `warmup` untimed ones; with a flush buffer (inputs that fit
    L2) every launch is timed alone after writing the buffer."""
    import torch

    for _ in range(warmup):
        fn()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    if flush is None:
        e[0].record(stream)
        for _ in range(steps):
            fn()
        e[1].record(stream)
        e[1].synchronize()
        return e[0].elapsed_time(e[1]) / steps
    total = 0.0
    for _ in range(steps):
        flush.zero_()
        e[0].record(stream)
        fn()
        e[1].record(stream)
        e[1].synchronize()
        total += e[0].elapsed_time(e[1])
    return total / steps


def single_config_leg(name, dev, stream, peak, steps, warmup, cpu_budget):
    """One of the single-problem configurations (C1, C3a, C3b) timed on the
    device, verified on the device, with its own roofline, clocks and CPU
    baseline."""
    import librett_gb300 as L

    prob = workload_problems(name, 1)[0]
    dims, perm, es = prob
    nb = problem_bytes(prob)
    d = DeviceData(dev, nb, 99)
    clocks = ClockSampler(dev.index or 0)
    with L.Plan(dims, perm, es, stream) as pl:
        run = lambda: pl.execute(d.inp.data_ptr(), d.out.data_ptr())  # noqa: E731
        clocks.start()
        ms = time_launches(run, stream, steps, warmup, d.flush)
        clk = clocks.stop()
        # back to back, as LibreTT's driver times (the comparison below): a
        # C-level loop of librettExecute calls on the plan
        # (librett_c_execute_batch), with no Python between the launches
        ms_b2b = ms
        if d.flush is not None:
            reps = 64
            loop = ([pl] * reps, [d.inp.data_ptr()] * reps, [d.out.data_ptr()] * reps)
            ms_b2b = time_launches(lambda: L.execute_batch(*loop), stream, steps, warmup) / reps
        bad, _ = L.verify(dims, perm, es, d.inp.data_ptr(), d.out.data_ptr(), stream)
        info = pl.info()
    gbs = 2 * nb / (ms / 1e3) / 1e9
    rec = {"workload": WORKLOADS[name], "bytes": nb, "ms": round(ms, 4), "gbs": round(gbs, 1),
           "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(gbs / peak, 4)},
           "method": L.METHOD_NAMES[info["method"]], "tile": info["tile_extent"],
           "verified": bad == 0, "clocks": clk,
           "l2": "flushed before every timed launch" if d.flush is not None else "inputs > L2"}
    if d.flush is not None:
        rec["gbs_back_to_back"] = round(2 * nb / (ms_b2b / 1e3) / 1e9, 1)
    if cpu_budget > 0:
        g, n, t = cpu_gather_time([prob], cpu_budget, host_threads())
        rec["cpu_baseline"] = {"value": round(g, 3), "unit": "GB/s", "cores": host_threads(),
                               "kind": "port", "sample": f"{n} host gather(s), {t:.2f} s"}
    del d
    return rec


LIBRETT_SUITE = 40  # suite problems LibreTT's build is timed on beside the engine


def librett_cuda_baseline(plan_cases, steps, warmup):
    """LibreTT's own CUDA build as a baseline (the reference's GPU path, not
    the thing measured): its unmodified sources compiled for sm_103a into
    oracle/_ref/ref_driver by build() where they are present, run as a
    separate process on this GPU through LibreTT's public API.  Times C1,
    C3a, C3b and the first LIBRETT_SUITE suite problems with librettPlan and
    with librettPlanMeasure (`steps` executes after `warmup`, CUDA events on
    the plan's stream), and the planning latency of both on plan_cases.
    Returns {"reason": ...} when the build is absent."""
    import tempfile

    drv = ROOT / "oracle" / "_ref" / "ref_driver"
    if not drv.exists():
        return {"reason": "LibreTT's CUDA build is absent on this machine: its sources were "
                          "not present when build() ran"}
    timed = ([("c1",) + tuple(workload_problems("c1", 1)[0]),
              ("c3a",) + tuple(workload_problems("c3a", 1)[0]),
              ("c3b",) + tuple(workload_problems("c3b", 1)[0])] +
             [(f"suite{i}",) + tuple(p) for i, p in enumerate(suite_problems()[:LIBRETT_SUITE])])

    def run(cases, st, wu, measure, env=None):
        with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
            for _, dims, perm, es in cases:
                f.write(" ".join(map(str, [len(dims), *dims, *perm, es, 2])) + "\n")
            path = f.name
        try:
            res = subprocess.run([str(drv), "bench", path, str(st), str(wu), str(measure)],
                                 capture_output=True, text=True, timeout=600,
                                 env=dict(os.environ, **(env or {})))
        finally:
            os.unlink(path)
        if res.returncode != 0:
            raise RuntimeError(f"LibreTT driver exit {res.returncode}: {res.stderr[-300:]}")
        return [json.loads(x) for x in res.stdout.splitlines() if x.startswith("{")]

    try:
        out = {"build": "LibreTT src/ unmodified, nvcc -O3 sm_103a (oracle/_ref/ref_driver)"}
        for measure, key in ((0, "plan"), (1, "plan_measure")):
            rows = run(timed, steps, warmup, measure)
            for (name, *_), r in zip(timed, rows):
                out.setdefault(name, {})[f"gbs_{key}"] = round(r["gbs"], 1)
            suite = [r["gbs"] for (name, *_), r in zip(timed, rows) if name.startswith("suite")]
            out.setdefault("suite40", {})[f"geomean_gbs_{key}"] = round(
                float(np.exp(np.mean(np.log(suite)))), 1)
        lat = {}
        for measure, key in ((0, "librettPlan"), (1, "librettPlanMeasure")):
            rows = run([("p",) + tuple(c) for c in plan_cases], 1, 0, measure)
            lat[key] = round(statistics.median(r["plan_ms"] for r in rows) * 1e3, 1)
        out["planning_us_median"] = lat
        return out
    except (RuntimeError, subprocess.TimeoutExpired, OSError) as e:
        return {"reason": f"LibreTT's CUDA build did not run: {e}"}


def grouped_leg(dev, stream, peak, steps, warmup, cpu_budget, nproblems=10000):
    """The batched configuration: 10,000 transposes as one grouped execution
    (one CUDA graph, the default tile policy) against the plain per-tensor
    librettExecute loop on the same buffers, both timed here; every member's
    output is then checked on the device."""
    import torch

    import librett_gb300 as L
    from librett_gb300.workloads import packed_offsets

    problems = workload_problems("grouped", nproblems)
    offs, total = packed_offsets(problems)
    d = DeviceData(dev, total, 4321)
    ins = [d.inp.data_ptr() + o for o in offs]
    outs = [d.out.data_ptr() + o for o in offs]
    t0 = time.perf_counter()
    plans = L.plan_batch(problems, stream)  # librettPlan on every member, one C call
    plan_s = time.perf_counter() - t0
    try:
        t0 = time.perf_counter()
        grp = L.Group(plans, ins, outs, stream)
        create_s = time.perf_counter() - t0
        ginfo = grp.info()
        clocks = ClockSampler(dev.index or 0)
        clocks.start()
        ms = time_launches(grp.execute, stream, steps, warmup)
        clk = clocks.stop()
        loop_ms = time_launches(lambda: L.execute_batch(plans, ins, outs), stream, steps, warmup)
        grp.execute()
        torch.cuda.synchronize(dev)
        ok = sum(L.verify(dd, p, es, i, o, stream)[0] == 0
                 for (dd, p, es), i, o in zip(problems, ins, outs))
        grp.destroy()
    finally:
        for pl in plans:
            pl.destroy()
    n = len(problems)
    gbs = ginfo["bytes"] / (ms / 1e3) / 1e9
    rec = {"workload": WORKLOADS["grouped"], "members": n, "bytes": ginfo["bytes"],
           "transposes_per_s": round(n / (ms / 1e3), 1), "ms": round(ms, 4), "gbs": round(gbs, 1),
           "loop": {"transposes_per_s": round(n / (loop_ms / 1e3), 1), "ms": round(loop_ms, 4),
                    "what": "librettExecute on every plan in turn"},
           "speedup_vs_loop": round(loop_ms / ms, 3),
           "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(gbs / peak, 4),
                        "basis": "algorithmic bytes of the group / graph time"},
           "buckets": ginfo["buckets"], "policy": "default (widest tiles, cp.async loads)",
           "plan_s": round(plan_s, 3), "group_create_s": round(create_s, 3),
           "verified": ok, "clocks": clk}
    if cpu_budget > 0:
        _, done, t = cpu_gather_time(problems, cpu_budget, host_threads())
        rec["cpu_baseline"] = {"value": round(done / t, 1), "unit": "transposes/s",
                               "cores": host_threads(), "kind": "port",
                               "sample": f"first {done} members, {t:.2f} s of host gather"}
    del d
    return rec


def planning_leg(dev, stream, cases):
    """Planning latency on held-out problems of the plan-selection
    distribution, each entry point in its own loop over the problems, as
    LibreTT's driver times its two planners:
    * librettPlan (learned selector, plan cache off) in a C-level loop
      (librett_c_plan_batch: the host duration of every librettPlan call
      measured inside the library's loop, no Python between the calls), alone
      and followed by a stream synchronise (LibreTT's driver synchronises
      after each plan); a plan of a tile with at most 6 ranks holds no device
      tables, a larger one writes its tables asynchronously, stream-ordered
      before any execute, so the plan is usable when the call returns;
    * the same librettPlan calls made one by one from Python (ctypes);
    * librettPlanMeasure (which synchronises internally) from Python: its
      0.5-1 ms make the call overhead negligible.
    Medians over the problems."""
    import ctypes

    import torch

    import librett_gb300 as L
    from librett_gb300 import _lib

    lib = _lib.load()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    maxb = max(problem_bytes(c) for c in cases)
    d = DeviceData(dev, maxb, 5)
    prev_sel = lib.librett_c_set_plan_selector(0)
    prev_cache = lib.librett_c_set_plan_cache(0)
    py_us, meas_us, learned = [], [], 0
    args = [(len(dims), _lib.int_array(dims), _lib.int_array(perm), es) for dims, perm, es in cases]
    try:
        loop_us = {}
        for sync in (False, True):
            torch.cuda.synchronize(dev)
            plans, us = L.plan_batch(cases, stream, synchronize=sync, timings=True)
            loop_us[sync] = us
            if not sync:
                learned = sum(pl.info()["selected_by"] == 1 for pl in plans)
            for pl in plans:
                pl.destroy()
        for rank, dc, pc, es in args:
            torch.cuda.synchronize(dev)
            h = ctypes.c_uint(0)
            t0 = time.perf_counter()
            rc = lib.librett_c_plan(ctypes.byref(h), rank, dc, pc, es, sptr)
            py_us.append((time.perf_counter() - t0) * 1e6)
            assert rc == 0, rc
            lib.librett_c_destroy(h.value)
        for rank, dc, pc, es in args:
            torch.cuda.synchronize(dev)
            h = ctypes.c_uint(0)
            t0 = time.perf_counter()
            rc = lib.librett_c_plan_measure(ctypes.byref(h), rank, dc, pc, es, sptr,
                                            d.inp.data_ptr(), d.out.data_ptr())
            meas_us.append((time.perf_counter() - t0) * 1e6)
            assert rc == 0, rc
            lib.librett_c_destroy(h.value)
    finally:
        lib.librett_c_set_plan_selector(prev_sel)
        lib.librett_c_set_plan_cache(prev_cache)
    a, b = statistics.median(loop_us[False]), statistics.median(meas_us)
    return {"problems": len(cases), "librettPlan_us_median": round(a, 1),
            "librettPlanMeasure_us_median": round(b, 1), "ratio": round(b / a, 2),
            "librettPlan_then_synchronize_us_median": round(statistics.median(loop_us[True]), 1),
            "librettPlan_from_python_us_median": round(statistics.median(py_us), 1),
            "ratio_from_python": round(b / statistics.median(py_us), 2),
            "learned_picks": learned,
            "how": "librettPlan: host duration of each call inside a C-level loop over the "
                   "problems (librett_c_plan_batch), plan cache off; librettPlanMeasure and "
                   "the from_python figures: duration of each C-ABI call from Python (ctypes); "
                   "each entry point in its own loop over the problems"}


def _time_candidate(pl, ip, op, stream, e):
    """Median of three event-timed batches of >= ~150 us of executes (ms)."""
    nb = problem_bytes((pl.dim, pl.permutation, pl.sizeofType))
    reps = int(min(64, max(1, np.ceil(150e-6 / (2.0 * nb / 5e12 + 4e-6)))))
    pl.execute(ip, op)
    ts = []
    for _ in range(3):
        e[0].record(stream)
        for _ in range(reps):
            pl.execute(ip, op)
        e[1].record(stream)
        e[1].synchronize()
        ts.append(e[0].elapsed_time(e[1]) / reps)
    return float(np.median(ts))


def selection_leg(dev, stream, cases):
    """Plan-choice regret on held-out problems: every candidate of the
    default set is timed, then the learned pick and the analytic pick are
    compared with the fastest (regret = t(pick) / t(best) - 1, geomean over
    problems)."""
    import ctypes

    import torch

    import librett_gb300 as L
    from librett_gb300 import _lib

    lib = _lib.load()
    maxb = max(problem_bytes(c) for c in cases)
    d = DeviceData(dev, maxb, 6)
    ip, op = d.inp.data_ptr(), d.out.data_ptr()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    prev_sel = lib.librett_c_set_plan_selector(0)
    prev_cache = lib.librett_c_set_plan_cache(0)
    ratios = {"learned": [], "analytic": []}
    try:
        for dims, perm, es in cases:
            picks = {}
            for mode, name in ((2, "learned"), (1, "analytic")):
                lib.librett_c_set_plan_selector(mode)
                with L.Plan(dims, perm, es, stream) as pl:
                    picks[name] = pl.info()["candidate"]
                    ncand = pl.info()["num_candidates"]
            lib.librett_c_set_plan_selector(0)
            times = []
            for c in range(ncand):
                with L.Plan(dims, perm, es, stream, candidate=c) as pl:
                    times.append(_time_candidate(pl, ip, op, stream, e))
            best = min(times)
            for name in ratios:
                ratios[name].append(times[picks[name]] / best)
    finally:
        lib.librett_c_set_plan_selector(prev_sel)
        lib.librett_c_set_plan_cache(prev_cache)
    g = {k: float(np.exp(np.mean(np.log(v)))) - 1 for k, v in ratios.items()}
    p90 = {k: float(np.percentile(v, 90)) - 1 for k, v in ratios.items()}
    return {"problems": len(cases),
            "regret_geomean": {k: round(v, 4) for k, v in g.items()},
            "regret_p90": {k: round(v, 4) for k, v in p90.items()},
            "exact_best": {k: int(sum(abs(x - 1) < 1e-9 for x in v)) for k, v in ratios.items()},
            "how": "every default candidate timed (median of 3 event-timed batches), "
                   "regret = t(pick)/t(best) - 1"}


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
    # inputs that fit L2: flush it before every launch, time the launches alone
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if maxb <= 256 << 20 else None

    def step(events=None):
        for k, pl in enumerate(plans):
            if flush is not None:
                flush.zero_()
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
    if flush is not None:  # the launches only, without the flushes between them
        ms = sum(e0.elapsed_time(e1) for evs in ev for e0, e1 in evs)
    ms_max = max_over_ranks(ms, world)
    value = world * step_bytes * args.steps / (ms_max / 1e3) / 1e9

    # every problem's output checked on the device (LibreTT's bench checks
    # every shape it times, tests/librett_bench.cpp:866)
    verified = None
    if not args.no_verify:
        verified = 0
        for (dims, perm, es), pl in zip(problems, plans):
            out.fill_(0xA5)
            pl.execute(ip, op)
            verified += L.verify(dims, perm, es, ip, op, stream)[0] == 0

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
    ceiling = copy_ceiling(inp, out, stream, (maxb // 8) * 8) if maxb >= 1 << 26 else None

    # end to end through the public API: pinned host in -> device -> host out.
    # The problems stream through two device buffer pairs: problem i + 1's
    # input copy (its own stream), problem i's transpose (the plans' stream)
    # and problem i - 1's result copy (a third stream) overlap, the two
    # copies in opposite directions of the host link.
    e2e = None
    if not args.no_e2e:
        hin = torch.empty(maxb, dtype=torch.uint8, pin_memory=True)
        hin.copy_(inp.cpu())
        hout = torch.empty(maxb, dtype=torch.uint8, pin_memory=True)
        d_in = [inp, torch.empty_like(inp)]
        d_out = [out, torch.empty_like(out)]
        s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        torch.cuda.synchronize(dev)

        def e2e_step():
            start = torch.cuda.Event()
            start.record(stream)
            s_in.wait_event(start)
            s_out.wait_event(start)
            loaded = [torch.cuda.Event() for _ in range(2)]
            done = [None, None]  # transpose of the buffer pair finished
            saved = [None, None]  # its result copied back
            for i, ((dims, perm, es), pl) in enumerate(zip(problems, plans)):
                b, nb = i % 2, problem_bytes((dims, perm, es))
                with torch.cuda.stream(s_in):
                    if done[b] is not None:
                        s_in.wait_event(done[b])
                    d_in[b][:nb].copy_(hin[:nb], non_blocking=True)
                    loaded[b].record(s_in)
                stream.wait_event(loaded[b])
                if saved[b] is not None:
                    stream.wait_event(saved[b])
                pl.execute(d_in[b].data_ptr(), d_out[b].data_ptr())
                done[b] = torch.cuda.Event()
                done[b].record(stream)
                with torch.cuda.stream(s_out):
                    s_out.wait_event(done[b])
                    hout[:nb].copy_(d_out[b][:nb], non_blocking=True)
                    saved[b] = torch.cuda.Event()
                    saved[b].record(s_out)
            for ev in saved:
                if ev is not None:
                    stream.wait_event(ev)

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
        if maxb >= 1 << 26:
            link = link_ceiling(hin, hout, d_in[1], d_out[1], maxb)
            link["e2e_frac_of_bidirectional"] = round(
                e2e["value"] / world / link["bidirectional_gbs"], 4)
            e2e["link_ceiling_same_run"] = link
        del hin, hout, d_in, d_out

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        gbs, n, t = cpu_gather_time(problems, args.cpu_budget, host_threads())
        cpu = {"value": round(gbs, 3), "unit": "GB/s", "cores": host_threads(), "kind": "port",
               "sample": f"first {n} problem(s) of the workload, {t:.1f} s of host gather"}

    # the other configurations, each timed and checked in this run (1 GPU)
    configs = None
    if args.workload == "suite" and world == 1 and not args.no_extras:
        for pl in plans:
            pl.destroy()
        plans = []
        del inp, out
        torch.cuda.empty_cache()
        suite_gbs = [2 * problem_bytes(p) / (t / 1e3) / 1e9 for p, t in zip(problems, per_problem_ms)]
        configs = extra_legs(args, dev, stream, peak, suite_gbs)

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
        "dtype": line_dtype(problems),
        "data": "synthetic random 64-bit patterns, fixed seeds",
        "config": workload_config(args, problems),
        "parallelism": f"replicas x{world}",
        "details": {"bytes_per_step": step_bytes, "candidate": args.candidate,
                    "methods": methods},
        "verified": verified,
        "geomean_gbs": round(geo, 3),
        "geomean_frac_of_copy": round(geo / peak, 4),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 3),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind,
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": d["bytes"] // d["launches"],
                     "copy_ceiling_same_run": ceiling},
        "per_kernel": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                           "gbs": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1)}
                       for k, v in per_kernel.items()},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "configs": configs,
    }
    print(json.dumps(line), flush=True)
    for pl in plans:
        pl.destroy()
    return 0


def extra_legs(args, dev, stream, peak, suite_gbs=None):
    """C1, C3a, C3b, the grouped batch, planning latency and plan-choice
    regret, each measured in this run, plus LibreTT's CUDA build on C1, C3a,
    C3b and the first suite problems when it is present."""
    from librett_gb300.learn.data import problems as selector_problems

    held_out = selector_problems(args.planning_problems, 424242)  # not used in training
    out = {}
    for name in ("c1", "c3a", "c3b"):
        out[name] = single_config_leg(name, dev, stream, peak, 20, 5, args.extra_cpu_budget)
    out["grouped"] = grouped_leg(dev, stream, peak, 5, 3, args.extra_cpu_budget,
                                 args.grouped_problems)
    out["planning"] = planning_leg(dev, stream, held_out)
    out["selection"] = selection_leg(dev, stream, held_out[:args.selection_problems])
    ref = librett_cuda_baseline(held_out, 10, 3)
    out["librett_cuda"] = ref
    if "reason" not in ref:
        for name in ("c1", "c3a", "c3b"):
            r = ref.get(name, {})
            # LibreTT's driver times launches back to back: compare like with like
            mine = out[name].get("gbs_back_to_back", out[name]["gbs"])
            if r.get("gbs_plan"):
                out[name]["vs_librett_plan"] = round(mine / r["gbs_plan"], 3)
                out[name]["vs_librett_plan_measure"] = round(mine / r["gbs_plan_measure"], 3)
        if suite_gbs is not None and len(suite_gbs) >= LIBRETT_SUITE and "suite40" in ref:
            mine = float(np.exp(np.mean(np.log(suite_gbs[:LIBRETT_SUITE]))))
            ref["suite40"]["engine_geomean_gbs"] = round(mine, 1)
            ref["suite40"]["vs_librett_plan"] = round(mine / ref["suite40"]["geomean_gbs_plan"], 3)
            ref["suite40"]["vs_librett_plan_measure"] = round(
                mine / ref["suite40"]["geomean_gbs_plan_measure"], 3)
        lat = ref.get("planning_us_median", {})
        if lat.get("librettPlanMeasure"):
            # LibreTT's driver times each plan call followed by a stream
            # synchronise: compare with the engine's plan-then-synchronise
            out["planning"]["vs_librett_plan_measure"] = round(
                lat["librettPlanMeasure"]
                / out["planning"]["librettPlan_then_synchronize_us_median"], 2)
    return out


def run_grouped(args):
    """Grouped workload: one step = one execution of a group of all the
    problems (one CUDA graph), each tensor at its own 256-byte-aligned offset
    of one input and one output buffer.  The plain per-tensor loop
    (librettExecute on every plan, one launch each) is timed on the same
    buffers in its own region."""
    import torch

    import librett_gb300 as L
    from librett_gb300.workloads import GROUPED_SEED, packed_offsets

    rank, local, world = dist_setup(args.gpus)
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    problems = workload_problems("grouped", args.problems)
    n = len(problems)
    offs, total = packed_offsets(problems)
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(4321 + rank)
    inp = torch.randint(-(2 ** 62), 2 ** 62, (total // 8,), dtype=torch.int64, device=dev,
                        generator=g).view(torch.uint8)
    out = torch.empty(total, dtype=torch.uint8, device=dev)
    ins = [inp.data_ptr() + o for o in offs]
    outs = [out.data_ptr() + o for o in offs]
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    plans = [L.Plan(d, p, es, stream) for d, p, es in problems]
    plan_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    grp = L.Group(plans, ins, outs, stream, policy=args.policy)
    create_s = time.perf_counter() - t0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def time_group(k):
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(k):
            grp.execute()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / k

    # the plan selector's tiles, then the autotuned tile policy (tuning is a
    # one-time cost per batch signature, outside the timed region)
    grp.execute()
    untuned_ms = time_group(max(1, args.steps))
    tune_s = None
    if not args.no_tune and args.policy is None:
        t0 = time.perf_counter()
        grp.tune()
        tune_s = time.perf_counter() - t0
    policy, tuned = grp.policy()
    ginfo = grp.info()
    if args.buckets:
        with open(args.buckets, "w") as fb:
            for b in grp.buckets():
                fb.write(json.dumps(b) + "\n")
    step_bytes = ginfo["bytes"]

    for _ in range(args.warmup):
        grp.execute()
        L.execute_batch(plans, ins, outs)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize(dev)
    launches0 = L.launch_count()
    e0.record(stream)
    for _ in range(args.steps):
        grp.execute()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    launches = L.launch_count() - launches0
    barrier(world)
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps

    # the plain per-tensor loop on the same buffers
    barrier(world)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(args.steps):
        L.execute_batch(plans, ins, outs)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    loop_ms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps

    value = world * n / (ms / 1e3)
    gbs = step_bytes / (ms / 1e3) / 1e9
    loop_value = world * n / (loop_ms / 1e3)
    peak, peak_kind = load_peaks()

    # end to end on a prefix of the batch whose inputs fit 2 GiB of pinned
    # host memory.  The prefix is cut into E2E_CHUNKS contiguous groups of
    # about equal bytes; chunk c + 1's input copy (own stream), group c
    # (the plans' stream) and chunk c - 1's output copy (a third stream)
    # overlap, the copies in opposite directions of the host link.
    e2e = None
    if not args.no_e2e:
        cap, m = 2 << 30, 0
        while m < n and offs[m] + problem_bytes(problems[m]) <= cap:
            m += 1
        sub_bytes = offs[m - 1] + problem_bytes(problems[m - 1])
        hin = torch.empty(sub_bytes, dtype=torch.uint8, pin_memory=True)
        hin.copy_(inp[:sub_bytes].cpu())
        hout = torch.empty(sub_bytes, dtype=torch.uint8, pin_memory=True)
        cuts = [0]
        for k in range(1, E2E_CHUNKS):
            want = sub_bytes * k / E2E_CHUNKS
            cuts.append(max(cuts[-1] + 1, next(i for i in range(m) if offs[i] >= want)))
        cuts.append(m)
        spans = []  # (first member, end member, first byte, end byte)
        for a, b in zip(cuts, cuts[1:]):
            spans.append((a, b, offs[a], offs[b - 1] + problem_bytes(problems[b - 1])))
        groups = [L.Group(plans[a:b], ins[a:b], outs[a:b], stream, policy=policy)
                  for a, b, _, _ in spans]
        s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        done = [None] * len(spans)   # group of the chunk finished (last step)
        saved = [None] * len(spans)  # its outputs copied back (last step)

        def e2e_step():
            start = torch.cuda.Event()
            start.record(stream)
            s_in.wait_event(start)
            s_out.wait_event(start)
            for c, ((_, _, lo, hi), grp) in enumerate(zip(spans, groups)):
                with torch.cuda.stream(s_in):
                    if done[c] is not None:
                        s_in.wait_event(done[c])
                    inp[lo:hi].copy_(hin[lo:hi], non_blocking=True)
                    loaded = torch.cuda.Event()
                    loaded.record(s_in)
                stream.wait_event(loaded)
                if saved[c] is not None:
                    stream.wait_event(saved[c])
                grp.execute()
                done[c] = torch.cuda.Event()
                done[c].record(stream)
                with torch.cuda.stream(s_out):
                    s_out.wait_event(done[c])
                    hout[lo:hi].copy_(out[lo:hi], non_blocking=True)
                    saved[c] = torch.cuda.Event()
                    saved[c].record(s_out)
            for ev in saved:
                stream.wait_event(ev)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize(dev)
        barrier(world)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ems = max_over_ranks(e0.elapsed_time(e1), world) / args.steps
        for grp in groups:
            grp.destroy()
        e2e = {"value": round(world * m / (ems / 1e3), 1), "unit": "transposes/s",
               "h2d_bytes_per_step": sub_bytes, "d2h_bytes_per_step": sub_bytes,
               "ms_per_step": round(ems, 3), "members": m, "chunks": len(spans),
               "note": f"first {m} problems of the batch (inputs within 2 GiB of pinned host "
                       f"memory) in {len(spans)} groups; each step copies every input in and "
                       "every output out, chunk copies overlapping the other chunks' groups"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        _, done, t = cpu_gather_time(problems, args.cpu_budget, host_threads())
        cpu = {"value": round(done / t, 1), "unit": "transposes/s", "cores": host_threads(),
               "kind": "port", "sample": f"first {done} problems of the batch, {t:.1f} s of "
                                         "host gather"}
    grp.destroy()
    for pl in plans:
        pl.destroy()
    if rank != 0:
        return 0
    line = {
        "metric": "transposes/s (grouped)",
        "value": round(value, 1),
        "unit": "transposes/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32/u64",
        "data": "synthetic random 64-bit patterns, fixed seeds",
        "config": {"workload": WORKLOADS["grouped"], "problems": n, "seed": GROUPED_SEED,
                   "bytes_per_step": step_bytes, "buckets": ginfo["buckets"],
                   "separate_members": ginfo["separate"], "tiles": ginfo["tiles"],
                   "l2": "inputs larger than L2, no flush",
                   "parallelism": f"replicas x{world}"},
        "gbs": round(gbs, 3),
        "loop": {"transposes_per_s": round(loop_value, 1), "ms_per_step": round(loop_ms, 4),
                 "gbs": round(step_bytes / (loop_ms / 1e3) / 1e9, 3),
                 "what": "librettExecute on every plan in turn (librett_c_execute_batch)"},
        "speedup_vs_loop": round(loop_ms / ms, 3),
        "untuned": {"ms_per_step": round(untuned_ms, 4),
                    "transposes_per_s": round(world * n / (untuned_ms / 1e3), 1),
                    "gbs": round(step_bytes / (untuned_ms / 1e3) / 1e9, 3)},
        "tile_policy": {"per_class": policy, "tuned": tuned,
                        "tune_s": None if tune_s is None else round(tune_s, 3),
                        "classes": "size class (<64KiB, <1MiB, <16MiB, larger) + 4 x element "
                                   "size (4, 8, 16 bytes)",
                        "values": "tile (0 selector, 1 wide, 2 widest, 3 full-device model) + 4 x "
                                  "loads (0 registers, 1 cp.async, 2 cp.async with persistent "
                                  "CTAs)"},
        "plan_s": round(plan_s, 3),
        "group_create_s": round(create_s, 3),
        "roofline": {"bound": "hbm", "kernel": "groupTileKernel", "achieved": round(gbs, 3),
                     "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
                     "peak_source": peak_kind, "traffic": None,
                     "basis": "algorithmic bytes of the whole group / graph time (the "
                              "buckets run concurrently)"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="suite")
    ap.add_argument("--problems", type=int, default=None,
                    help="problems of the workload (suite: 200, grouped: 10000)")
    ap.add_argument("--cpu-budget", type=float, default=12.0,
                    help="seconds of host gather for the cpu_baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-verify", action="store_true",
                    help="skip the device check of every problem's output after timing")
    ap.add_argument("--no-extras", action="store_true",
                    help="suite workload: skip the other configurations (C1, C3a, C3b, grouped, "
                         "planning, selection, LibreTT's CUDA build)")
    ap.add_argument("--extra-cpu-budget", type=float, default=2.0,
                    help="seconds of host gather for each extra configuration's cpu_baseline")
    ap.add_argument("--selection-problems", type=int, default=100,
                    help="held-out problems whose every candidate is timed for the regret")
    ap.add_argument("--planning-problems", type=int, default=200,
                    help="held-out problems of the plan-selection distribution for planning latency")
    ap.add_argument("--grouped-problems", type=int, default=10000,
                    help="members of the batched configuration in the suite line's extras")
    ap.add_argument("--buckets", type=str, default=None,
                    help="grouped workload: write the graph's bucket launches (JSON lines)")
    ap.add_argument("--policy", type=str, default=None,
                    help="grouped workload: policy for all classes, per size class (4 values) or per "
                         "class (12 values), e.g. 6 or 0,1,1,0 (no tuning)")
    ap.add_argument("--no-tune", action="store_true",
                    help="grouped workload: keep the plan selector's tiles (no autotuning)")
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
    if args.policy is not None:
        args.policy = [int(x) for x in args.policy.split(",")]
    if args.problems is None:
        args.problems = 10000 if args.workload == "grouped" else 200
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "grouped":
        return run_grouped(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())
