"""Host-side checks of the bulk-copy tile pipeline (no GPU).

A bulk-copy tile (pipeline 3) loads each contiguous segment of its input
with one cp.async.bulk: a segment must be one piece of global memory and
one piece of shared memory, 16-byte aligned in both, and the segments must
cover the tile.  librett_c_bulk_check verifies that on the host, from the
same offset tables the flat kernel reads, for a candidate of the planner's
full candidate set.
"""
import numpy as np

import bench
from librett_gb300 import _lib
from librett_gb300.learn.data import problems as selector_problems
from tests import shapes as S

LIBRETT_SUCCESS, LIBRETT_INVALID_PARAMETER, LIBRETT_INVALID_DEVICE = 0, 2, 3


def _check(dims, perm, es):
    lib = _lib.load()
    dc, pc = _lib.int_array(dims), _lib.int_array(perm)
    n = 0
    for cand in range(64):
        rc = lib.librett_c_bulk_check(len(dims), dc, pc, es, 152, cand)
        if rc == LIBRETT_INVALID_PARAMETER:
            break
        assert rc in (LIBRETT_SUCCESS, LIBRETT_INVALID_DEVICE), (dims, perm, es, cand, rc)
        n += rc == LIBRETT_SUCCESS
    return n


def _all_pipelines(fn):
    lib = _lib.load()
    prev = lib.librett_c_set_candidate_set(1)
    try:
        return fn()
    finally:
        lib.librett_c_set_candidate_set(prev)


def test_bulk_segments_suite_and_selector_distribution():
    def run():
        n = sum(_check(d, p, es) for d, p, es in bench.suite_problems(200))
        n += sum(_check(d, p, es) for d, p, es in selector_problems(400, 9))
        return n
    assert _all_pipelines(run) > 300


def test_bulk_segments_random_high_rank():
    rng = np.random.default_rng(12)

    def run():
        n = 0
        for _ in range(300):
            dims, perm, es = S.random_problem(rng, max_rank=10, max_vol=1 << 22)
            n += _check(dims, perm, es)
        return n
    assert _all_pipelines(run) > 50


def test_bulk_in_the_default_candidate_set():
    """The default candidate set holds the bulk-copy twin of flat tiles whose
    segments allow it (C3a's input runs are 1.5 KB), and the check passes
    there too."""
    lib = _lib.load()
    prev = lib.librett_c_set_candidate_set(0)
    try:
        dims, perm, es = S.C3A
        assert _check(list(dims), list(perm), es) >= 1
        n = sum(_check(d, p, es) for d, p, es in bench.suite_problems(60))
        assert n > 30
    finally:
        lib.librett_c_set_candidate_set(prev)
