"""Host-side checks of grouped execution (no GPU).

The grouped kernel addresses a tile through run tables (one entry per
contiguous input or output run plus the position inside the run) instead of
the single-plan kernel's per-unit tables.  librett_c_group_run_check runs the
kernel's index arithmetic on the host for every unit of a candidate tile and
compares it with the per-unit tables, which the planner tests already check
against the oracle's coverage.  Also: the batch generator's distribution.
"""
import numpy as np
import pytest

from librett_gb300 import _lib
from librett_gb300.workloads import grouped_problems, packed_offsets
from tests import shapes as S

LIBRETT_SUCCESS, LIBRETT_INVALID_PARAMETER, LIBRETT_INVALID_DEVICE = 0, 2, 3


def _check_all_candidates(dims, perm, es):
    lib = _lib.load()
    dc, pc = _lib.int_array(dims), _lib.int_array(perm)
    checked = 0
    for cand in range(16):
        for element_units in (0, 1):
            rc = lib.librett_c_group_run_check(len(dims), dc, pc, es, 152, cand, element_units)
            if rc == LIBRETT_INVALID_PARAMETER:
                return checked  # no more candidates
            assert rc in (LIBRETT_SUCCESS, LIBRETT_INVALID_DEVICE), (dims, perm, es, cand, rc)
            checked += rc == LIBRETT_SUCCESS
    return checked


def test_run_tables_batch_distribution():
    n = 0
    for dims, perm, es in grouped_problems(600, seed=7, log2_lo=4, log2_hi=22, sizes=(4, 8, 16)):
        n += _check_all_candidates(dims, perm, es)
    assert n > 2000


def test_run_tables_random_high_rank():
    rng = np.random.default_rng(8)
    n = 0
    for _ in range(300):
        dims, perm, es = S.random_problem(rng, max_rank=12, max_vol=1 << 22)
        n += _check_all_candidates(dims, perm, es)
    assert n > 500


@pytest.mark.parametrize("dims,perm,es", [S.C1, S.C3A, S.C3B, (S.EXAMPLE[0], S.EXAMPLE[1], 8),
                                          ([3] * 16, list(range(15, -1, -1)), 4),
                                          ([2, 3] * 8, [0, 2, 4, 6, 8, 10, 12, 14, 1, 3, 5, 7, 9,
                                                        11, 13, 15], 8)])
def test_run_tables_named_shapes(dims, perm, es):
    assert _check_all_candidates(list(dims), list(perm), es) > 0


def test_grouped_distribution():
    probs = grouped_problems(2000)
    ranks = np.array([len(d) for d, _, _ in probs])
    vols = np.array([np.prod(d, dtype=np.float64) for d, _, _ in probs])
    sizes = np.array([es for _, _, es in probs])
    assert ranks.min() == 2 and ranks.max() == 6
    assert vols.min() >= 2 ** 10 * 0.9 and vols.max() <= 2 ** 22 * 1.1
    assert 0.45 < np.mean(sizes == 4) < 0.55
    assert all(sorted(p) == list(range(len(d))) for d, p, _ in probs)
    offs, total = packed_offsets(probs)
    assert all(o % 256 == 0 for o in offs) and total >= offs[-1] + vols[-1] * sizes[-1]


def test_run_division_identity():
    """The grouped kernel divides in-tile indices n < 2^16 by run lengths
    d < 2^16 as umulhi(n + 1, floor((2^32 - 1) / d)) (RunDiv in plan.h).
    Exhaustive over n for every d up to 4096 and 2,000 larger d, including
    powers of two and the largest values."""
    n = np.arange(1 << 16, dtype=np.uint64)
    rng = np.random.default_rng(3)
    ds = list(range(1, 4097)) + [1 << k for k in range(12, 16)] + [65535, 65534, 65533]
    ds += rng.integers(4097, 65536, 2000).tolist()
    for d in ds:
        mul = np.uint64(0xFFFFFFFF // d)
        q = ((n + np.uint64(1)) * mul) >> np.uint64(32)
        assert np.array_equal(q, n // np.uint64(d)), d
