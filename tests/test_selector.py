"""Learned plan selection, host side (CPU only): the host inference the
planner runs, the weight file, its rejection rules and the fallback to the
analytic model."""
import ctypes
import os

import numpy as np
import pytest

import librett_gb300 as L
from librett_gb300 import _lib
from librett_gb300.learn import data as D
from librett_gb300.learn import train as T
from oracle import mlp_oracle as M

NF = _lib.load().librett_c_mlp_feature_count()


@pytest.fixture
def restore_selector():
    lib = _lib.load()
    prev = lib.librett_c_set_plan_selector(0)
    lib.librett_c_set_plan_selector(prev)
    yield lib
    lib.librett_c_set_plan_selector(prev)
    lib.librett_c_load_plan_model(None)


def _fp(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def test_sizes():
    lib = _lib.load()
    assert lib.librett_c_mlp_feature_count() == NF
    assert lib.librett_c_mlp_param_count() == 128 * NF + 128 + 2 * (128 * 128 + 128) + 128 + 1


def test_host_inference_matches_float64_oracle():
    lib = _lib.load()
    rng = np.random.default_rng(0)
    params = T.init_params(NF, rng)
    params[-129:-1] *= 10  # make the output layer matter
    X = rng.normal(size=(50, NF)).astype(np.float32)
    p, pp = _fp(params)
    x, xp = _fp(X)
    out = np.zeros(50, dtype=np.float32)
    assert lib.librett_c_mlp_predict_host(pp, xp, 50,
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    ref, _ = M.forward(params, X)
    assert np.allclose(out, ref, rtol=1e-4, atol=1e-4)


def _predict(lib, pp, X):
    x, xp = _fp(X)
    out = np.zeros(len(x), dtype=np.float32)
    assert lib.librett_c_mlp_predict_host(pp, xp, len(x),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    return out


def test_host_inference_does_not_depend_on_row_grouping():
    """The host inference leaves out hidden inputs that are zero in every row
    of a row block; a row's prediction is bit-identical whether it is scored
    alone or in a batch with rows of other zero patterns (near-duplicate rows,
    like the candidates of one problem, share most of their zeros)."""
    lib = _lib.load()
    rng = np.random.default_rng(5)
    params = T.init_params(NF, rng)
    params[-129:-1] *= 10
    _, pp = _fp(params)
    base = rng.normal(size=(8, NF))
    X = np.concatenate([b + 0.05 * rng.normal(size=(6, NF)) for b in base]).astype(np.float32)
    whole = _predict(lib, pp, X)
    alone = np.array([_predict(lib, pp, X[i:i + 1])[0] for i in range(len(X))], dtype=np.float32)
    assert np.array_equal(whole.view(np.uint32), alone.view(np.uint32))
    for n in range(1, 10):  # the planner's short-list sizes, every block split
        order = rng.permutation(len(X))[:n]
        got = _predict(lib, pp, X[order])
        assert np.array_equal(got.view(np.uint32), whole[order].view(np.uint32)), n
    ref, _ = M.forward(params, X)
    assert np.allclose(whole, ref, rtol=1e-4, atol=1e-4)


def test_features_finite_and_deterministic():
    for dims, perm, es in D.problems(30, seed=3):
        n = L.describe(dims, perm, es)["num_candidates"]
        for c in range(n):
            f1 = D.features(dims, perm, es, c)
            f2 = D.features(dims, perm, es, c)
            assert f1.shape == (NF,) and np.all(np.isfinite(f1)) and np.array_equal(f1, f2)


def _write(tmp_path, sms=152, device="", corrupt=None):
    rng = np.random.default_rng(1)
    params = T.init_params(NF, rng)
    path = str(tmp_path / "m.bin")
    T.save_model(path, params, np.zeros(NF, np.float32), np.ones(NF, np.float32), 0.0, 1.0, sms,
                 device)
    if corrupt == "byte":
        raw = bytearray(open(path, "rb").read())
        raw[200] ^= 0xFF
        open(path, "wb").write(bytes(raw))
    elif corrupt == "truncate":
        raw = open(path, "rb").read()
        open(path, "wb").write(raw[:-100])
    elif corrupt == "nan":
        params[5] = np.nan
        T.save_model(path, params, np.zeros(NF, np.float32), np.ones(NF, np.float32), 0.0, 1.0,
                     sms, device)
    return path, params


def test_model_file_round_trip(tmp_path):
    path, params = _write(tmp_path)
    m = T.load_model(path)
    assert np.array_equal(m["params"], params.astype(np.float32))


@pytest.mark.parametrize("corrupt", ["byte", "truncate", "nan"])
def test_bad_model_files_rejected(tmp_path, restore_selector, corrupt):
    lib = restore_selector
    path, _ = _write(tmp_path, corrupt=corrupt)
    assert lib.librett_c_load_plan_model(path.encode()) == L.LIBRETT_INVALID_PARAMETER
    assert lib.librett_c_load_plan_model(str(tmp_path / "missing.bin").encode()) != 0


def test_learned_used_when_loaded_and_fallback_otherwise(tmp_path, restore_selector):
    lib = restore_selector
    dims, perm, es = [64, 48, 32], [2, 0, 1], 4
    path, _ = _write(tmp_path, sms=152)
    assert lib.librett_c_load_plan_model(path.encode()) == 0
    lib.librett_c_set_plan_selector(0)
    assert L.describe(dims, perm, es, num_sms=152)["selected_by"] == 1
    # a model for another SM count does not apply
    assert L.describe(dims, perm, es, num_sms=132)["selected_by"] == 0
    # forced analytic
    lib.librett_c_set_plan_selector(1)
    assert L.describe(dims, perm, es, num_sms=152)["selected_by"] == 0
    # a single-candidate problem needs no model
    lib.librett_c_set_plan_selector(2)
    assert L.describe([5, 7], [0, 1], 8, num_sms=152)["selected_by"] == 0
    assert lib.librett_c_set_plan_selector(7) == -1


def test_learned_pick_is_argmin_of_predictions_over_short_list(tmp_path, restore_selector):
    """The analytic model short-lists the candidates of its 4 cheapest tiles
    (ties by index; a tile's per-unit and bulk-copy variants count once, and
    only the SHORTLIST_TWINS cheapest tiles keep the bulk-copy variant, when
    their input runs hold at least SHORTLIST_TWIN_MIN_RUN bytes); the learned
    pick is the lowest prediction among those."""
    lib = restore_selector
    path, params = _write(tmp_path, sms=152)
    assert lib.librett_c_load_plan_model(path.encode()) == 0
    lib.librett_c_set_plan_selector(2)
    for dims, perm, es in D.problems(10, seed=11):
        n = L.describe(dims, perm, es)["num_candidates"]
        X = np.stack([D.features(dims, perm, es, c) for c in range(n)])
        pred, _ = M.forward(params, X)
        infos = [L.describe(dims, perm, es, candidate=c) for c in range(n)]
        order = sorted(range(n), key=lambda c: infos[c]["model_cost"])
        key = [tuple(i["tile_extent"]) if i["method"] in (2, 3, 4) else ("kernel", c)
               for c, i in enumerate(infos)]
        tiles, short = [], []
        for c in order:
            if key[c] not in tiles:
                if len(tiles) == 4:
                    break
                tiles.append(key[c])
            if infos[c]["pipeline"] == 3 and (
                    tiles.index(key[c]) >= T.SHORTLIST_TWINS or
                    2.0 ** (X[c, T.RUN_IN_COL] * 20) < T.SHORTLIST_TWIN_MIN_RUN - 0.5):
                continue
            short.append(c)
        got = L.describe(dims, perm, es)["candidate"]
        assert got in short
        best = pred[short].min()
        assert pred[got] <= best + 1e-4 * max(1.0, abs(best))


def test_shortlist_regret_rules():
    """Deployed-selection regret: persistent-pipeline candidates are outside
    the default set, the short list is the k lowest analytic costs, the pick
    the lowest score on it, regret against the set's best."""
    X = np.zeros((5, NF), dtype=np.float32)
    X[:, T.COST_COL] = [0.1, 0.2, 0.3, 0.4, 0.0]
    X[:, 12] = [1, 2, 3, 4, 5]  # five different tiles
    X[4, T.PIPE_REG_COL] = 1  # cheapest and fastest, but not a default candidate
    t = np.array([3.0, 2.0, 1.5, 1.0, 0.5])
    prob = np.zeros(5, dtype=int)
    score = np.array([5.0, 4.0, 3.0, 0.0, -1.0])
    assert T.shortlist_regret(score, X, t, prob, 0)[0] == 0.0  # picks candidate 3
    assert T.shortlist_regret(score, X, t, prob, 3)[0] == 0.5  # 2 of {0, 1, 2}: 1.5 / 1.0
    assert T.shortlist_regret(score, X, t, prob, 1)[0] == 2.0  # only 0: 3.0 / 1.0
    # a bulk-copy twin of tile 0 (same tile columns) joins the short list of 1
    X[:, T.RUN_IN_COL] = np.log2(4096) / 20  # input runs of 4 KiB
    X2 = np.concatenate([X, X[:1]])
    X2[5, T.BULK_COL] = 1
    t2 = np.concatenate([t, [1.2]])
    score2 = np.concatenate([score, [4.5]])
    prob2 = np.zeros(6, dtype=int)
    assert abs(T.shortlist_regret(score2, X2, t2, prob2, 1)[0] - 0.2) < 1e-12
    # ... but not when the tile's input runs are shorter than the threshold
    X2s = X2.copy()
    X2s[:, T.RUN_IN_COL] = np.log2(512) / 20
    assert T.shortlist_regret(score2, X2s, t2, prob2, 1)[0] == 2.0
    assert abs(T.shortlist_regret(score2, X2s, t2, prob2, 1, min_run=0)[0] - 0.2) < 1e-12
    # a twin of the third-cheapest tile stays off the short list
    X3 = np.concatenate([X, X[2:3]])
    X3[5, T.BULK_COL] = 1
    t3 = np.concatenate([t, [0.6]])
    score3 = np.concatenate([score, [-5.0]])
    assert T.shortlist_regret(score3, X3, t3, prob2, 3, twins=2)[0] == 1.5 / 0.6 - 1.0  # picks 2
    assert T.shortlist_regret(score3, X3, t3, prob2, 3, twins=3)[0] == 0.0


def test_targets_relative_and_clipped():
    t = np.array([1.0, 2.0, 100.0, 3.0, 3.0])
    prob = np.array([0, 0, 0, 1, 1])
    y = T.targets(t, prob)
    assert y[0] == 0 and abs(y[1] - np.log(2)) < 1e-12 and y[2] == T.Y_CLIP and y[3] == y[4] == 0


def test_timing_file_merges_large_sets():
    """The committed timing file packs the base set and any number of
    large-problem sets; problem indices of later sets are renumbered."""
    import json

    def ds(problems, prob, t):
        return {"problems": np.array(json.dumps(problems)), "prob": np.array(prob),
                "cand": np.array([0] * len(prob)), "t": np.array(t), "sms": np.array(152),
                "device": np.array("d")}

    a = ds([[[4, 4], [1, 0], 8]], [0, 0], [1.0, 2.0])
    b = ds([[[8, 2], [1, 0], 4], [[3, 5], [1, 0], 16]], [0, 1, 1], [3.0, 4.0, 5.0])
    m = D.merge_datasets([a, b])
    assert json.loads(str(m["problems"])) == [[[4, 4], [1, 0], 8], [[8, 2], [1, 0], 4],
                                              [[3, 5], [1, 0], 16]]
    assert m["prob"].tolist() == [0, 0, 1, 2, 2] and m["t"].tolist() == [1.0, 2.0, 3.0, 4.0, 5.0]
    packed = D.pack_timings(a, m)
    assert packed["large_prob"].tolist() == [0, 0, 1, 2, 2]
    assert packed["prob"].tolist() == [0, 0]
