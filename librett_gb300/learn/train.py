"""Train the plan-selection MLP on the GPU with the library's own kernels.

Targets: for candidate c of problem p with measured time t[c],
    y = min(log(t[c] / min_c' t[c']), 1.5)
i.e. the log slowdown against the problem's fastest candidate, clipped so
that very poor candidates do not dominate the loss (only the ranking near
the best matters).  Features and targets are standardised; the
standardisation is stored in the weight file and applied by the library at
plan time.  Loss: mean squared error.  Optimiser: Adam.  Every forward,
backward, loss and update step runs in librett_c_mlp_* kernels; torch only
holds the device buffers and gathers mini-batches.

Usage (on a GPU):
    python -m librett_gb300.learn.train --data data.npz --holdout 1000 \\
        [--extra large.npz] --out librett_gb300/models/plan_mlp.bin --report report.json
"""
from __future__ import annotations

import argparse
import ctypes
import json
import struct
import sys

import numpy as np

from .. import _lib

MAGIC = b"LTMLPv01"
HIDDEN, LAYERS = 128, 4
Y_CLIP = 1.5


def fnv1a(data: bytes) -> int:
    h = 2166136261
    for b in data:
        h ^= b
        h = (h * 16777619) & 0xFFFFFFFF
    return h


def save_model(path, params, mean, std, ymean, ystd, sms, device):
    lib = _lib.load()
    nfeat = lib.librett_c_mlp_feature_count()
    npar = lib.librett_c_mlp_param_count()
    assert params.size == npar and mean.size == nfeat and std.size == nfeat
    body = MAGIC + struct.pack("<4I", nfeat, HIDDEN, LAYERS, npar) + struct.pack("<i", int(sms))
    body += device.encode()[:63].ljust(64, b"\0")
    body += np.concatenate([mean, std, [ymean, ystd], params]).astype("<f4").tobytes()
    body += struct.pack("<I", fnv1a(body))
    with open(path, "wb") as f:
        f.write(body)


def load_model(path):
    raw = open(path, "rb").read()
    nfeat, hid, lay, npar = struct.unpack("<4I", raw[8:24])
    vals = np.frombuffer(raw[92:-4], dtype="<f4")
    return {"mean": vals[:nfeat], "std": vals[nfeat:2 * nfeat], "ymean": float(vals[2 * nfeat]),
            "ystd": float(vals[2 * nfeat + 1]), "params": vals[2 * nfeat + 2:].copy()}


def targets(t, prob):
    y = np.empty_like(t)
    for p in np.unique(prob):
        m = prob == p
        y[m] = np.minimum(np.log(t[m] / t[m].min()), Y_CLIP)
    return y


def init_params(nfeat, rng):
    def w(o, i):
        return rng.normal(0.0, np.sqrt(2.0 / i), (o, i))
    parts = [w(HIDDEN, nfeat), np.zeros(HIDDEN), w(HIDDEN, HIDDEN), np.zeros(HIDDEN),
             w(HIDDEN, HIDDEN), np.zeros(HIDDEN), w(1, HIDDEN) * 0.1, np.zeros(1)]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


class GpuMlp:
    """Device buffers and the kernel calls of one training run."""

    def __init__(self, params: np.ndarray, max_batch: int):
        import torch

        self.torch = torch
        lib = _lib.load()
        self.lib = lib
        self.n = params.size
        self.p = torch.from_numpy(params.astype(np.float32)).cuda()
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.ws = torch.zeros(lib.librett_c_mlp_workspace_floats(max_batch), device="cuda")
        self.out = torch.zeros(max_batch, device="cuda")
        self.dout = torch.zeros(max_batch, device="cuda")
        self.loss = torch.zeros(1, device="cuda")
        self.stream = torch.cuda.current_stream().cuda_stream
        self.step = 0

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with {rc}")

    def forward(self, X):
        b = X.shape[0]
        self._check(self.lib.librett_c_mlp_forward(self.p.data_ptr(), X.data_ptr(), b,
                                                   self.ws.data_ptr(), self.out.data_ptr(),
                                                   self.stream), "forward")
        return self.out[:b]

    def train_step(self, X, y, lr):
        b = X.shape[0]
        self.forward(X)
        self._check(self.lib.librett_c_mlp_mse_grad(self.out.data_ptr(), y.data_ptr(), b,
                                                    self.dout.data_ptr(), self.loss.data_ptr(),
                                                    self.stream), "mse_grad")
        self._check(self.lib.librett_c_mlp_backward(self.p.data_ptr(), X.data_ptr(), b,
                                                    self.ws.data_ptr(), self.dout.data_ptr(),
                                                    self.g.data_ptr(), self.stream), "backward")
        self.step += 1
        self._check(self.lib.librett_c_mlp_adam(self.p.data_ptr(), self.g.data_ptr(),
                                                self.m.data_ptr(), self.v.data_ptr(), self.n,
                                                ctypes.c_float(lr), ctypes.c_float(0.9),
                                                ctypes.c_float(0.999), ctypes.c_float(1e-8),
                                                self.step, self.stream), "adam")

    def gradients(self, X, y):
        """Loss and gradients of one batch (no update) -- for the gradient check."""
        b = X.shape[0]
        self.loss.zero_()
        self.forward(X)
        self.lib.librett_c_mlp_mse_grad(self.out.data_ptr(), y.data_ptr(), b, self.dout.data_ptr(),
                                        self.loss.data_ptr(), self.stream)
        self.lib.librett_c_mlp_backward(self.p.data_ptr(), X.data_ptr(), b, self.ws.data_ptr(),
                                        self.dout.data_ptr(), self.g.data_ptr(), self.stream)
        self.torch.cuda.synchronize()
        return float(self.loss.item()), self.g.cpu().numpy().copy()

    def params(self):
        return self.p.cpu().numpy().copy()


def predict_host(params, Xs):
    """The library's host inference (the planner's own), for standardised
    rows Xs."""
    lib = _lib.load()
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(Xs, dtype=np.float32)
    out = np.zeros(x.shape[0], dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    rc = lib.librett_c_mlp_predict_host(p.ctypes.data_as(fp), x.ctypes.data_as(fp), x.shape[0],
                                        out.ctypes.data_as(fp))
    if rc != 0:
        raise RuntimeError(f"librett_c_mlp_predict_host: {rc}")
    return out


def predict_gpu(params, Xs, batch=4096):
    import torch

    net = GpuMlp(params, batch)
    out = []
    for i in range(0, Xs.shape[0], batch):
        xb = torch.from_numpy(np.ascontiguousarray(Xs[i:i + batch], dtype=np.float32)).cuda()
        out.append(net.forward(xb).cpu().numpy().copy())
    return np.concatenate(out)


def train(X, y, epochs=60, batch=1024, lr=2e-3, seed=0, log=True):
    """Returns (params, mean, std, ymean, ystd, loss history)."""
    import torch

    rng = np.random.default_rng(seed)
    mean = X.mean(0)
    std = X.std(0)
    std[std < 1e-6] = 1.0
    ymean, ystd = float(y.mean()), float(y.std() or 1.0)
    Xs = ((X - mean) / std).astype(np.float32)
    ys = ((y - ymean) / ystd).astype(np.float32)
    Xd = torch.from_numpy(Xs).cuda()
    yd = torch.from_numpy(ys).cuda()
    net = GpuMlp(init_params(X.shape[1], rng), batch)
    hist = []
    n = Xs.shape[0]
    for ep in range(epochs):
        order = torch.from_numpy(rng.permutation(n)).cuda()
        lr_ep = lr * (0.5 * (1 + np.cos(np.pi * ep / epochs)))  # cosine schedule
        net.loss.zero_()
        nb = 0
        for i in range(0, n, batch):
            idx = order[i:i + batch]
            net.train_step(Xd.index_select(0, idx).contiguous(), yd.index_select(0, idx).contiguous(),
                           lr_ep)
            nb += 1
        torch.cuda.synchronize()
        hist.append(float(net.loss.item()) / nb)
        if log and (ep % 10 == 0 or ep == epochs - 1):
            print(f"  epoch {ep:3d}  lr {lr_ep:.2e}  loss {hist[-1]:.4f}", flush=True)
    return net.params(), mean.astype(np.float32), std.astype(np.float32), ymean, ystd, hist


def choice_regret(score, t, prob):
    """Per problem: measured time of the lowest-score candidate / best - 1."""
    reg = []
    for p in np.unique(prob):
        m = np.nonzero(prob == p)[0]
        pick = m[np.argmin(score[m])]
        reg.append(t[pick] / t[m].min() - 1.0)
    return np.array(reg)


def geo_regret(reg):
    return float(np.exp(np.mean(np.log1p(reg))) - 1.0)


# Feature columns (librett_gb300/csrc/select.cpp planFeatures): 9 and 10 mark
# the persistent pipelines, which are not in the default candidate set; 30 is
# the analytic model's cost (log scale, monotone in it); 32 marks a bulk-copy
# variant, which shares its tile (and the columns below) with a per-unit one.
PIPE_REG_COL, PIPE_ASYNC_COL, COST_COL, BULK_COL = 9, 10, 30, 32
TILE_COLS = [8, 12, 13, 14, 15, 16, 17, 18, 30]


SHORTLIST_TWINS = 4  # short-listed tiles that keep their bulk-copy twin
SHORTLIST_TWIN_MIN_RUN = 2048  # ... when their input runs hold this many bytes
RUN_IN_COL = 14  # log2(input run bytes) / 20


def shortlist_regret(score, X, t, prob, k, twins=SHORTLIST_TWINS, min_run=SHORTLIST_TWIN_MIN_RUN):
    """Regret of the deployed selection, per problem: within the default
    candidate set, the lowest score among the candidates of the analytic
    model's k cheapest tiles (a tile's per-unit and bulk-copy variants count
    once, and only the `twins` cheapest tiles keep the bulk-copy variant,
    when their input runs hold at least `min_run` bytes; k <= 0: among all),
    against the set's measured best."""
    default = (X[:, PIPE_REG_COL] == 0) & (X[:, PIPE_ASYNC_COL] == 0)
    reg = []
    for p in np.unique(prob):
        m = np.nonzero((prob == p) & default)[0]
        if len(m) == 0:
            continue
        keep = m[np.argsort(X[m, COST_COL], kind="stable")]
        if k > 0:
            tiles, short = [], []
            for i in keep:
                key = tuple(X[i, TILE_COLS])
                if key not in tiles:
                    if len(tiles) == k:
                        break
                    tiles.append(key)
                if X[i, BULK_COL] == 1 and (tiles.index(key) >= twins or
                                            2.0 ** (X[i, RUN_IN_COL] * 20) < min_run - 0.5):
                    continue
                short.append(i)
            keep = np.array(short, dtype=keep.dtype)
        pick = keep[np.argmin(score[keep])]
        reg.append(t[pick] / t[m].min() - 1.0)
    return np.array(reg)


def evaluate_model(d, model, holdout):
    """Held-out and training regret of a saved model on a dataset, with the
    planner's short lists (host inference, no GPU needed)."""
    X, t, prob = d["X"], d["t"], d["prob"]
    split = int(prob.max()) + 1 - holdout
    pred = predict_host(model["params"], (X - model["mean"]) / model["std"])
    rep = {}
    for name, mask in (("train", prob < split), ("holdout", prob >= split)):
        r = {}
        for k in (0, 4, 3, 2):
            reg = shortlist_regret(pred[mask], X[mask], t[mask], prob[mask], k)
            r[f"shortlist_{k or 'all'}"] = {"geomean_regret": geo_regret(reg),
                                             "p90_regret": float(np.quantile(reg, 0.9)),
                                             "problems": int(len(reg))}
        rep[name] = r
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--data", required=True)
    ap.add_argument("--holdout", type=int, default=1000, help="last N problems are held out")
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--out", default=None)
    ap.add_argument("--report", default=None)
    ap.add_argument("--evaluate", default=None, metavar="MODEL",
                    help="no training: report the regret of this saved model over the default "
                         "candidate set, ranking all candidates or the analytic short list of 4 "
                         "or 3 (host inference)")
    ap.add_argument("--extra", action="append", default=[],
                    help="further datasets used for training only (e.g. larger problems)")
    args = ap.parse_args(argv)
    d = np.load(args.data)
    if args.evaluate:
        rep = evaluate_model(d, load_model(args.evaluate), args.holdout)
        print(json.dumps(rep, indent=1))
        if args.report:
            with open(args.report, "w") as f:
                json.dump(rep, f, indent=1)
        return 0
    if args.out is None:
        ap.error("--out is required when training")
    X, t, prob, cand = d["X"], d["t"], d["prob"], d["cand"]
    heur = d["heuristic"]
    nprob = int(prob.max()) + 1
    split = nprob - args.holdout
    tr, te = prob < split, prob >= split
    y = targets(t, prob)
    Xtr, ytr = X[tr], y[tr]
    extra_problems = 0
    for path in args.extra:
        e = np.load(path)
        Xtr = np.concatenate([Xtr, e["X"]])
        ytr = np.concatenate([ytr, targets(e["t"], e["prob"])])
        extra_problems += int(e["prob"].max()) + 1
    params, mean, std, ymean, ystd, hist = train(Xtr, ytr, epochs=args.epochs)
    save_model(args.out, params, mean, std, ymean, ystd, int(d["sms"]), str(d["device"]))
    pred = predict_gpu(params, (X - mean) / std) * ystd + ymean
    rep = {"train_problems": int(split), "extra_train_problems": extra_problems,
           "holdout_problems": int(args.holdout), "rows": int(len(t)), "final_loss": hist[-1]}
    for name, mask in (("train", tr), ("holdout", te)):
        r_mlp = choice_regret(pred[mask], t[mask], prob[mask])
        # analytic model: its pick per problem
        r_ana = []
        for p in np.unique(prob[mask]):
            m = np.nonzero(prob == p)[0]
            pick = m[cand[m] == heur[p]][0]
            r_ana.append(t[pick] / t[m].min() - 1.0)
        r_ana = np.array(r_ana)
        rep[name] = {"mlp_geomean_regret": geo_regret(r_mlp),
                     "analytic_geomean_regret": geo_regret(r_ana),
                     "mlp_p90_regret": float(np.quantile(r_mlp, 0.9)),
                     "analytic_p90_regret": float(np.quantile(r_ana, 0.9)),
                     "mlp_exact_best_frac": float(np.mean(r_mlp == 0.0))}
    print(json.dumps(rep, indent=1))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(rep, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
