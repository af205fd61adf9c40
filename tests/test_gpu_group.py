"""Grouped execution (librettGroup* / librettExecuteGrouped) against the oracle.

Many uneven transposes share one input and one output buffer, each tensor at
its own offset with a canary-filled gap behind it.  After the group runs,
every tensor must equal the oracle's transpose bit for bit and every gap must
still hold the canary.  Covered: mixed ranks, permutations and element sizes
(4/8/16 bytes); members whose pointers are not 16-byte aligned (element
units inside their bucket); members whose tile extent the grouped planner
rounds so that their runs take 16-byte units; 4-byte members in 16-byte
units with tiles of twice the single-plan volume; a rank-16 member with
many grid ranks; a second
execution after the inputs changed (the graph reads the buffers anew); plans
destroyed before the group runs; every tile and load policy (persistent
CTAs included) and the autotuner; the
one-shot librettExecuteGrouped; the plain per-tensor loop; and the error
codes.
"""
import numpy as np
import pytest

import librett_gb300 as L
from librett_gb300.workloads import grouped_problems
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CANARY = 0x5A
GAP = 64


def _layout(problems, misalign):
    """Byte offsets: 256-aligned starts plus, for members flagged in
    `misalign`, a shift by one element (4 or 8 bytes), or by the given
    number of bytes where the flag is an int."""
    offs, total = [], 0
    for (dims, _, es), mis in zip(problems, misalign):
        shift = mis if type(mis) is int else (es if mis else 0)
        start = total + shift
        offs.append(start)
        nb = int(np.prod(dims)) * es
        total = (start + nb + GAP + 255) // 256 * 256
    return offs, total


def _mixed_problems(n, seed):
    probs = grouped_problems(n, seed=seed, log2_lo=4, log2_hi=15, sizes=(4, 8, 16), max_rank=6)
    probs.append(([2, 3] * 8, [int(x) for x in np.random.default_rng(seed).permutation(16)], 4))
    probs.append(([5], [0], 8))                      # rank 1: a plain copy
    probs.append(([7, 1, 9, 1], [3, 2, 1, 0], 16))   # unit dims fuse away
    return probs


class _Batch:
    def __init__(self, probs, misalign, seed):
        import torch

        self.probs = probs
        self.offs, total = _layout(probs, misalign)
        self.total = total
        self.rng = np.random.default_rng(seed)
        self.inp = torch.zeros(total, dtype=torch.uint8, device="cuda")
        self.out = torch.full((total,), CANARY, dtype=torch.uint8, device="cuda")
        self.host = None
        self.refill()

    def refill(self):
        import torch

        self.host = self.rng.integers(0, 256, self.total, dtype=np.uint8)
        self.inp.copy_(torch.from_numpy(self.host))

    def ptrs(self):
        return ([self.inp.data_ptr() + o for o in self.offs],
                [self.out.data_ptr() + o for o in self.offs])

    def check(self):
        import torch

        torch.cuda.synchronize()
        res = self.out.cpu().numpy()
        covered = np.zeros(self.total, dtype=bool)
        for i, ((dims, perm, es), o) in enumerate(zip(self.probs, self.offs)):
            nb = int(np.prod(dims)) * es
            want = O.transpose_np(self.host[o:o + nb], dims, perm, es).view(np.uint8)
            got = res[o:o + nb]
            if not np.array_equal(got, want):
                bad = int(np.nonzero(got != want)[0][0])
                raise AssertionError(f"member {i} dims {dims} perm {perm} es {es}: byte {bad}")
            covered[o:o + nb] = True
        assert (res[~covered] == CANARY).all(), "write outside the members' outputs"


def _plans(probs, stream):
    return [L.Plan(d, p, es, stream) for d, p, es in probs]


def test_group_mixed_bit_exact(cuda):
    import torch

    probs = _mixed_problems(400, seed=11)
    rng = np.random.default_rng(5)
    misalign = [bool(rng.random() < 0.15) and es < 16 for _, _, es in probs]
    b = _Batch(probs, misalign, seed=3)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    before = L.launch_count()
    with L.Group(plans, ins, outs, stream) as g:
        info = g.info()
        assert info["members"] == len(probs)
        assert info["bytes"] == sum(2 * int(np.prod(d)) * es for d, _, es in probs)
        launches = L.launch_count()
        g.execute()
        assert L.launch_count() - launches == info["buckets"] + info["separate"]
        b.check()
        b.refill()
        g.execute()
        b.check()
    for p in plans:
        p.destroy()
    assert L.launch_count() > before


def test_group_f32_eight_byte_units(cuda):
    """4-byte elements move in 8-byte units on the sides whose runs or
    pointers allow 8 but not 16 bytes (members shifted by 8 bytes are 8- but
    not 16-byte aligned); such buckets exist and every member is bit-exact."""
    import torch

    probs = grouped_problems(300, seed=23, log2_lo=4, log2_hi=15, sizes=(4,), max_rank=6)
    rng = np.random.default_rng(7)
    shifts = [8 if rng.random() < 0.3 else 0 for _ in probs]
    b = _Batch(probs, shifts, seed=9)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, stream) as g:
        units = {(k["lv"], k["sv"]) for k in g.buckets() if k["es"] == 4}
        assert any(2 in u for u in units), units
        assert units <= {(a, c) for a in (1, 2, 4) for c in (1, 2, 4)}, units
        g.execute()
        b.check()
    for p in plans:
        p.destroy()


def test_group_extent_rounding_widens_units(cuda):
    """8-byte elements whose picked tile has odd runs on both sides (9 x 151
    x 3, 15 x 13 x 21): the grouped planner rounds one extent to an even
    count (the last tile of the rank shifts back to end at the dim), so the
    runs take 16-byte units; the outputs are bit-exact."""
    import torch

    probs = [([9, 131028, 3], [2, 1, 0], 8), ([15, 13, 102, 2], [0, 2, 1, 3], 8)]
    b = _Batch(probs, [0, 0], seed=17)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, stream) as g:
        units = {(k["es"], k["lv"], k["sv"]) for k in g.buckets()}
        assert units == {(8, 2, 2)}, units
        g.execute()
        b.check()
    for p in plans:
        p.destroy()


def test_group_doubles_float32_tiles(cuda):
    """4-byte elements in 16-byte units get tiles of up to 8192 elements
    (8 load units per thread, 32 KB) in a group, twice the single-plan
    limit; the outputs are bit-exact."""
    import torch

    probs = [([64, 256, 64], [2, 0, 1], 4), ([128, 96, 40], [1, 2, 0], 4),
             ([32, 48, 20, 12], [3, 1, 0, 2], 4)]
    b = _Batch(probs, [0, 0, 0], seed=19)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, stream) as g:
        shapes = {(k["es"], k["lv"], k["sv"], k["nl"]) for k in g.buckets()}
        assert shapes == {(4, 4, 4, 8)}, shapes
        g.execute()
        b.check()
    for p in plans:
        p.destroy()


def test_group_high_rank_member(cuda):
    import torch

    # 16 unfusable ranks: every flat tile leaves nine or more grid ranks,
    # whose decode the group does once per tile at creation
    probs = [([3] * 16, list(range(15, -1, -1)), 4)] + _mixed_problems(20, seed=21)
    b = _Batch(probs, [False] * len(probs), seed=9)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, stream) as g:
        assert g.info()["separate"] == 0
        g.execute()
        b.check()
    for p in plans:
        p.destroy()


@pytest.mark.parametrize("policy", [(0, 0, 0, 0), (1, 1, 1, 1), (2, 2, 2, 2), (3, 3, 3, 3),
                                    (4, 4, 4, 4), (5, 5, 5, 5), (6, 6, 6, 6), (7, 7, 7, 7),
                                    (8, 8, 8, 8), (9, 9, 9, 9), (10, 10, 10, 10),
                                    (11, 11, 11, 11), (2, 4, 3, 5), (6, 0, 7, 1), (7, 1, 4, 2),
                                    (10, 1, 6, 11)])
def test_group_policies(cuda, policy):
    import torch

    probs = _mixed_problems(150, seed=16)
    rng = np.random.default_rng(17)
    misalign = [bool(rng.random() < 0.2) and es < 16 for _, _, es in probs]
    b = _Batch(probs, misalign, seed=10)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, stream, policy=policy) as g:
        assert g.policy() == (L.expand_policy(policy), False)
        g.execute()
        b.check()
    for p in plans:
        p.destroy()


def test_group_tune_and_cache(cuda):
    import torch

    probs = grouped_problems(300, seed=18, log2_lo=10, log2_hi=18)
    b = _Batch(probs, [False] * len(probs), seed=11)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, stream) as g:
        g.tune()
        pol, tuned = g.policy()
        assert tuned and all(0 <= x < 12 for x in pol)
        b.out.fill_(CANARY)
        g.execute()
        b.check()
    # a new group over the same batch starts from the tuned policy
    with L.Group(plans, ins, outs, stream) as g2:
        assert g2.policy() == (pol, True)
    for p in plans:
        p.destroy()


def test_group_outlives_its_plans(cuda):
    import torch

    probs = _mixed_problems(120, seed=12)
    b = _Batch(probs, [False] * len(probs), seed=4)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    g = L.Group(plans, ins, outs, stream)
    for p in plans:
        p.destroy()
    g.execute()
    b.check()
    g.destroy()


def test_group_on_side_stream(cuda):
    import torch

    probs = _mixed_problems(60, seed=13)
    b = _Batch(probs, [False] * len(probs), seed=6)
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    plans = _plans(probs, side)
    ins, outs = b.ptrs()
    with L.Group(plans, ins, outs, side) as g:
        g.execute()
        side.synchronize()
        b.check()
    for p in plans:
        p.destroy()


def test_execute_grouped_one_shot(cuda):
    import torch

    probs = _mixed_problems(80, seed=14)
    b = _Batch(probs, [False] * len(probs), seed=7)
    plans = _plans(probs, torch.cuda.current_stream())
    ins, outs = b.ptrs()
    L.execute_grouped(plans, ins, outs)
    b.check()
    for p in plans:
        p.destroy()


def test_execute_batch_loop(cuda):
    import torch

    probs = _mixed_problems(80, seed=15)
    b = _Batch(probs, [False] * len(probs), seed=8)
    plans = _plans(probs, torch.cuda.current_stream())
    ins, outs = b.ptrs()
    L.execute_batch(plans, ins, outs)
    b.check()
    for p in plans:
        p.destroy()


def test_group_errors(cuda):
    import ctypes

    import torch

    lib = L._lib.load()
    s = torch.cuda.current_stream()
    buf = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    out = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    with L.Plan([8, 16], [1, 0], 4, s) as p:
        with pytest.raises(L.LibrettError) as e:
            L.Group([p], [buf.data_ptr()], [buf.data_ptr()], s)
        assert e.value.code == L.LIBRETT_INVALID_PARAMETER
        with pytest.raises(L.LibrettError) as e:
            L.Group([p], [buf.data_ptr() + 2], [out.data_ptr()], s)  # not 4-byte aligned
        assert e.value.code == L.LIBRETT_INVALID_PARAMETER
        with pytest.raises(L.LibrettError) as e:
            L.Group([123456789], [buf.data_ptr()], [out.data_ptr()], s)
        assert e.value.code == L.LIBRETT_INVALID_PLAN
        # members must be independent: an output overlapping another member's
        # input or output is rejected; shared inputs are fine (512 B tensors)
        for ins, outs in (([0, 1024], [2048, 2048 + 256]),    # outputs overlap
                          ([0, 2048 + 508], [2048, 3072]),    # output under an input
                          ([0, 1024], [1024 + 100, 2048])):   # output over an input
            with pytest.raises(L.LibrettError) as e:
                L.Group([p, p], [buf.data_ptr() + i for i in ins],
                        [buf.data_ptr() + o for o in outs], s)
            assert e.value.code == L.LIBRETT_INVALID_PARAMETER, (ins, outs)
        with L.Group([p, p], [buf.data_ptr(), buf.data_ptr() + 256],
                     [out.data_ptr(), out.data_ptr() + 512], s) as g:
            g.execute()
        with pytest.raises(L.LibrettError) as e:
            L.execute_batch([p, p], [buf.data_ptr(), buf.data_ptr()],
                            [out.data_ptr(), buf.data_ptr()])
        assert e.value.code == L.LIBRETT_INVALID_PARAMETER
    h = ctypes.c_uint(0)
    assert lib.librett_c_group_create(ctypes.byref(h), 0, None, None, None,
                                      ctypes.c_void_p(s.cuda_stream)) == L.LIBRETT_INVALID_PARAMETER
    assert lib.librett_c_group_execute(987654) == L.LIBRETT_INVALID_PLAN
    assert lib.librett_c_group_destroy(987654) == L.LIBRETT_INVALID_PLAN
    assert lib.librett_c_execute_grouped(0, None, None, None) == L.LIBRETT_INVALID_PARAMETER
    assert lib.librett_c_group_tune(987654) == L.LIBRETT_INVALID_PLAN
    with L.Plan([8, 16], [1, 0], 4, s) as p:
        with pytest.raises(L.LibrettError) as e:
            L.Group([p], [buf.data_ptr()], [out.data_ptr()], s, policy=(0, 0, 12, 0))
        assert e.value.code == L.LIBRETT_INVALID_PARAMETER


def test_group_execute_while_tuning(cuda):
    # one thread executes the group while another tunes it (the tuner
    # rebuilds the graph); every execution must see a complete graph
    import threading

    import torch

    probs = _mixed_problems(120, seed=19)
    b = _Batch(probs, [False] * len(probs), seed=12)
    stream = torch.cuda.current_stream()
    plans = _plans(probs, stream)
    ins, outs = b.ptrs()
    errors = []
    with L.Group(plans, ins, outs, stream) as g:
        def runner():
            try:
                for _ in range(50):
                    g.execute()
            except Exception as e:  # reported below
                errors.append(e)

        t = threading.Thread(target=runner)
        t.start()
        g.tune()
        t.join()
        assert not errors, errors
        b.out.fill_(CANARY)
        g.execute()
        b.check()
    for p in plans:
        p.destroy()
