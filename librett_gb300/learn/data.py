"""Problems and per-candidate timings for the learned plan selector.

Problem distribution: rank uniform in 2..7; volume log-uniform in
2^16..2^28 bytes; element size uniform in {4, 8, 16}; dims drawn
log-uniformly (random weights summing to log2 volume, each dim >= 2);
uniformly random permutation.

Timing of one candidate: plan it (librett_c_plan_candidate), one untimed
launch, then three batches of R back-to-back launches between CUDA events on
the plan's stream (R chosen so a batch lasts about 100 us, 1 <= R <= 64); the
time is the median batch time / R.

Usage (on a GPU):
    python -m librett_gb300.learn.data --problems 6000 --seed 7 --out data.npz
Recomputing the features of a collected dataset (host only):
    python -m librett_gb300.learn.data --refeature data.npz --out data2.npz
Both datasets from the committed timings (host only; writes data.npz and
data_large.npz):
    python -m librett_gb300.learn.data \
        --from-timings librett_gb300/models/plan_timings_gb300.npz --out data.npz
Packing collected datasets (base distribution, then one or more
large-problem supplements, merged) into a timing file of that form (host
only):
    python -m librett_gb300.learn.data --pack data.npz data_large.npz [more_large.npz ...] \
        --out librett_gb300/models/plan_timings_gb300.npz
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
import time

import numpy as np

from .. import _lib
import librett_gb300 as L

MIN_LOG2_BYTES, MAX_LOG2_BYTES = 16, 28


def problems(n: int, seed: int, min_log2_bytes: float = MIN_LOG2_BYTES,
             max_log2_bytes: float = MAX_LOG2_BYTES):
    """n random problems (dims, perm, element bytes) of the selector's distribution
    (or of the same distribution over another byte range)."""
    rng = np.random.Generator(np.random.MT19937(seed))
    out = []
    while len(out) < n:
        rank = int(rng.integers(2, 8))
        es = int(rng.choice([4, 8, 16]))
        logbytes = rng.uniform(min_log2_bytes, max_log2_bytes)
        logvol = logbytes - np.log2(es)
        if logvol < rank:  # every dim >= 2
            continue
        w = rng.uniform(0.05, 1.0, rank)
        logd = w / w.sum() * logvol
        dims = [max(2, int(round(2.0 ** x))) for x in logd]
        while int(np.prod(dims)) * es > 2 ** max_log2_bytes:
            i = int(np.argmax(dims))
            dims[i] = max(2, dims[i] // 2)
        perm = [int(x) for x in rng.permutation(rank)]
        out.append((dims, perm, es))
    return out


def features(dims, perm, es, candidate, num_sms=152):
    nf = _lib.load().librett_c_mlp_feature_count()
    buf = (ctypes.c_float * nf)()
    rc = _lib.load().librett_c_candidate_features(len(dims), _lib.int_array(dims),
                                                  _lib.int_array(perm), es, num_sms, candidate,
                                                  buf, nf)
    if rc != L.LIBRETT_SUCCESS:
        raise L.LibrettError(rc, "librett_c_candidate_features")
    return np.frombuffer(buf, dtype=np.float32).copy()


def time_candidate(dims, perm, es, candidate, stream, din, dout, ev):
    import torch

    plan = L.Plan(dims, perm, es, stream, candidate=candidate)
    try:
        nbytes = int(np.prod(dims)) * es
        est = 2.0 * nbytes / 5e12 + 4e-6
        reps = int(min(64, max(1, np.ceil(100e-6 / est))))
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
    finally:
        plan.destroy()


def collect(probs, num_sms, log_every=200):
    """Times every candidate of every problem; returns the dataset dict."""
    import torch

    stream = torch.cuda.current_stream()
    maxb = max(int(np.prod(d)) * es for d, _, es in probs)
    a = torch.empty(maxb, dtype=torch.uint8, device="cuda")
    b = torch.empty(maxb, dtype=torch.uint8, device="cuda")
    a.random_(0, 256)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    X, T, P, C = [], [], [], []
    heur, nbytes = [], []
    t0 = time.time()
    for i, (dims, perm, es) in enumerate(probs):
        h = L.describe(dims, perm, es, num_sms=num_sms)
        for c in range(h["num_candidates"]):
            X.append(features(dims, perm, es, c, num_sms))
            T.append(time_candidate(dims, perm, es, c, stream, a.data_ptr(), b.data_ptr(), ev))
            P.append(i)
            C.append(c)
        heur.append(h["candidate"])  # the analytic model's pick (selector forced to analytic)
        nbytes.append(int(np.prod(dims)) * es)
        if log_every and (i + 1) % log_every == 0:
            print(f"  {i + 1}/{len(probs)} problems, {len(T)} candidates, {time.time() - t0:.0f} s",
                  flush=True)
    return {"X": np.array(X, dtype=np.float32), "t": np.array(T), "prob": np.array(P),
            "cand": np.array(C), "heuristic": np.array(heur), "bytes": np.array(nbytes),
            "problems": json.dumps(probs)}


def refeature(d):
    """Recompute the features and the analytic model's picks of a dataset
    from its problems and candidate indices with the current library (the
    timings stay; candidates are numbered as with every pipeline on)."""
    lib = _lib.load()
    probs = [tuple(x) for x in json.loads(str(d["problems"]))]
    sms = int(d["sms"])
    prev_sel = lib.librett_c_set_plan_selector(1)
    prev_set = lib.librett_c_set_candidate_set(1)
    try:
        X = np.stack([features(*probs[int(p)], int(c), sms) for p, c in zip(d["prob"], d["cand"])])
        heur = np.array([L.describe(dims, perm, es, num_sms=sms)["candidate"]
                         for dims, perm, es in probs])
    finally:
        lib.librett_c_set_candidate_set(prev_set)
        lib.librett_c_set_plan_selector(prev_sel)
    out = {k: d[k] for k in d}
    out["X"] = X.astype(np.float32)
    out["heuristic"] = heur
    return out


def from_timings(path):
    """The two datasets (base distribution, large-problem supplement) of a
    committed timing file (librett_gb300/models/plan_timings_*.npz), with
    features computed by the current library."""
    z = np.load(path)
    base = {"problems": z["problems"], "prob": z["prob"], "cand": z["cand"], "t": z["t"],
            "sms": z["sms"], "device": z["device"]}
    large = {"problems": z["large_problems"], "prob": z["large_prob"], "cand": z["large_cand"],
             "t": z["large_t"], "sms": z["sms"], "device": z["device"]}
    return refeature(base), refeature(large)


def merge_datasets(parts):
    """One dataset of several collected ones (problem indices renumbered):
    problems, candidate indices and times."""
    problems, prob, cand, t = [], [], [], []
    for d in parts:
        prob.append(np.asarray(d["prob"]) + len(problems))
        problems += json.loads(str(d["problems"]))
        cand.append(np.asarray(d["cand"]))
        t.append(np.asarray(d["t"]))
    return {"problems": np.array(json.dumps(problems)), "prob": np.concatenate(prob),
            "cand": np.concatenate(cand), "t": np.concatenate(t), "sms": parts[0]["sms"],
            "device": parts[0]["device"]}


def pack_timings(base, large):
    """The committed timing-file form of two collected datasets: problems,
    candidate indices and times only (features are recomputed on load)."""
    return {"problems": base["problems"], "prob": base["prob"], "cand": base["cand"],
            "t": base["t"], "large_problems": large["problems"], "large_prob": large["prob"],
            "large_cand": large["cand"], "large_t": large["t"], "sms": base["sms"],
            "device": base["device"]}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--problems", type=int, default=6000)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--min-log2-bytes", type=float, default=MIN_LOG2_BYTES)
    ap.add_argument("--max-log2-bytes", type=float, default=MAX_LOG2_BYTES)
    ap.add_argument("--out", required=True)
    ap.add_argument("--refeature", default=None,
                    help="recompute features of this dataset (no GPU needed) instead of timing")
    ap.add_argument("--from-timings", default=None,
                    help="build both datasets from a committed timing file (no GPU needed)")
    ap.add_argument("--pack", nargs="+", default=None, metavar="BASE LARGE",
                    help="write the timing file of collected datasets: the base distribution, "
                         "then one or more large-problem supplements, merged (no GPU needed)")
    args = ap.parse_args(argv)
    if args.pack:
        if len(args.pack) < 2:
            ap.error("--pack needs BASE and at least one LARGE dataset")
        zb = np.load(args.pack[0])
        large = [np.load(f) for f in args.pack[1:]]
        out = pack_timings({k: zb[k] for k in zb.files},
                           merge_datasets([{k: z[k] for k in z.files} for z in large]))
        np.savez_compressed(args.out, **out)
        print(f"wrote {args.out}: {len(out['t'])} + {len(out['large_t'])} timings")
        return 0
    if args.refeature:
        z = np.load(args.refeature)
        data = refeature({k: z[k] for k in z.files})
        np.savez_compressed(args.out, **data)
        print(f"wrote {args.out}: {len(data['t'])} rows")
        return 0
    if args.from_timings:
        base, large = from_timings(args.from_timings)
        stem = args.out[:-4] if args.out.endswith(".npz") else args.out
        np.savez_compressed(args.out, **base)
        np.savez_compressed(stem + "_large.npz", **large)
        print(f"wrote {args.out} ({len(base['t'])} rows) and {stem}_large.npz "
              f"({len(large['t'])} rows)")
        return 0
    import torch

    torch.cuda.set_device(0)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    prev = _lib.load().librett_c_set_plan_selector(1)  # heuristic picks = the analytic model
    _lib.load().librett_c_set_candidate_set(1)  # time every pipeline
    probs = problems(args.problems, args.seed, args.min_log2_bytes, args.max_log2_bytes)
    data = collect(probs, sms)
    _lib.load().librett_c_set_plan_selector(prev)
    data["sms"] = sms
    data["device"] = torch.cuda.get_device_properties(0).name
    np.savez_compressed(args.out, **data)
    print(f"wrote {args.out}: {len(data['t'])} rows, {len(probs)} problems")
    return 0


if __name__ == "__main__":
    sys.exit(main())
