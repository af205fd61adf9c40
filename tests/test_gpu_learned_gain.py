"""What the trained network gains over the analytic model it replaces.

On problems of the selector's distribution drawn with a seed not used in
training, plans chosen by the learned model (the default when its weight
file is present) must run faster than plans chosen by the analytic model,
geomean over the problems, and must not be a large loss on any one of them
(relative for launches of 10 us or more, absolute below).
"""
import numpy as np
import pytest

import librett_gb300 as L
from librett_gb300 import _lib
from librett_gb300.learn.data import problems
from librett_gb300.learn.evaluate import evaluate

pytestmark = pytest.mark.gpu


def test_learned_choice_beats_analytic(cuda):
    lib = _lib.load()
    assert lib.librett_c_load_plan_model(None) == L.LIBRETT_SUCCESS, "weight file missing"
    # 80 problems across the whole distribution (2^16..2^28 bytes); every
    # execute time is the median of three batches of at least ~200 us
    probs = problems(80, seed=97531)
    summary, rows = evaluate(probs)
    # every problem with more than one candidate (plain copies have one)
    multi = sum(L.describe(r["dims"], r["perm"], r["es"])["num_candidates"] > 1 for r in rows)
    assert summary["learned_used"] == multi
    ratio = summary["exec_time_ratio_learned_over_analytic_geomean"]
    print("learned / analytic execute time, geomean:", ratio)
    # measured 0.986 on one GB300 (the analytic model's picks are within 5 %
    # of the best on average, the network's within 2 %); timing noise on the
    # geomean of 80 problems is about 0.2 %
    assert ratio < 0.995
    # no large loss on any one problem: at most 25 % where the analytic pick
    # runs 10 us or longer; below that a launch is latency-bound (the
    # candidates of a 2^16-byte problem run 4-6 us), so the loss is bounded
    # in time instead (3 us)
    for r in rows:
        la, an = r["exec_ms_learned"], r["exec_ms_analytic"]
        if an >= 0.010:
            assert la / an < 1.25, r
        else:
            assert la - an < 0.003, r
