"""Plan tables come from a host-side arena with stream-ordered reuse.

Only tiles of more than 6 ranks keep offset tables (smaller tiles compute
their addresses in the kernel), so every problem here is a rank-9..11 one
planned with a candidate that holds tables (checked through table_bytes).

A plan destroyed while kernels that read its tables are still queued on its
stream must keep those tables intact until the stream has passed the
destroy: plans created meanwhile on another stream get other memory, while a
plan on the same stream may take the block at once (stream order runs its
table writes after the queued kernels).  The stream is kept busy by a long
run of device copies queued ahead of the transposes, so the plans on the
second stream are created and executed while the first stream's transposes
are still waiting.  Every output stays bit-exact.
"""
import numpy as np
import pytest

import librett_gb300 as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tabled(dims, perm, es):
    """A candidate of the problem whose tile keeps offset tables (more than 6
    tile ranks), whatever the selector would pick."""
    n = L.describe(dims, perm, es)["num_candidates"]
    for c in range(n):
        if L.describe(dims, perm, es, candidate=c)["table_bytes"] > 0:
            return c
    raise AssertionError(("no candidate with tables", dims, perm, es))


def _plan(dims, perm, es, stream):
    return L.Plan(dims, perm, es, stream, candidate=_tabled(dims, perm, es))


def _problem(dims, perm, es, seed):
    _tabled(dims, perm, es)
    host = np.random.default_rng(seed).integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
    return host, O.transpose_np(host, dims, perm, es).view(np.uint8)


def test_reuse_waits_for_the_freeing_stream(cuda):
    import torch

    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    es = 4
    dims_a, perm_a = [4, 2, 4, 2, 2, 3, 2, 4, 2, 2, 2], [9, 6, 3, 7, 1, 0, 8, 10, 5, 2, 4]
    host_a, want_a = _problem(dims_a, perm_a, es, 1)
    inp_a = torch.from_numpy(host_a).cuda()
    outs_a = [torch.zeros_like(inp_a) for _ in range(4)]
    # other problems, other tables, the same range of table sizes
    others = [([2, 2, 4, 2, 2, 2, 3, 2, 4, 2, 2], [10, 6, 1, 3, 0, 8, 9, 2, 4, 7, 5]),
              ([2, 2, 2, 2, 3, 2, 2, 2, 2, 4, 2], [2, 10, 8, 6, 1, 4, 7, 9, 5, 3, 0]),
              ([2, 3, 2, 2, 2, 2, 2, 3, 4, 2], [9, 8, 6, 5, 7, 4, 1, 3, 0, 2]),
              ([4, 2, 2, 2, 3, 2, 4, 4, 2, 2], [5, 6, 9, 0, 2, 1, 7, 3, 8, 4]),
              ([4, 2, 4, 3, 2, 2, 2, 3, 3, 3], [5, 4, 7, 0, 9, 2, 6, 1, 3, 8]),
              ([2, 2, 2, 4, 4, 2, 3, 2, 2, 2], [5, 3, 0, 7, 9, 1, 6, 2, 8, 4])]
    ins_b, wants_b = [], []
    for k, (d, p) in enumerate(others):
        h, w = _problem(d, p, es, 10 + k)
        ins_b.append(torch.from_numpy(h).cuda())
        wants_b.append(w)
    outs_b = [torch.zeros_like(t) for t in ins_b]
    busy_src = torch.empty(1 << 29, dtype=torch.uint8, device="cuda")
    busy_dst = torch.empty_like(busy_src)
    torch.cuda.synchronize()

    with torch.cuda.stream(s1):
        for _ in range(40):  # tens of milliseconds of copies ahead of the transposes
            busy_dst.copy_(busy_src)
        plan_a = _plan(dims_a, perm_a, es, s1)
        for k in range(16):
            plan_a.execute(inp_a.data_ptr(), outs_a[k % 4].data_ptr())
        plan_a.destroy()  # its transposes are still queued behind the copies
        # the same stream may reuse the block at once
        plan_c = _plan(others[0][0], others[0][1], es, s1)
        out_c = torch.zeros_like(ins_b[0])
        plan_c.execute(ins_b[0].data_ptr(), out_c.data_ptr())
    assert s1.query() is False, "the first stream finished too early for this test to mean anything"
    plans_b = []
    for k, (d, p) in enumerate(others):
        pb = _plan(d, p, es, s2)
        pb.execute(ins_b[k].data_ptr(), outs_b[k].data_ptr())
        plans_b.append(pb)
    torch.cuda.synchronize()
    plan_c.destroy()
    for pb in plans_b:
        pb.destroy()
    torch.cuda.synchronize()

    for o in outs_a:
        assert np.array_equal(o.cpu().numpy(), want_a)
    assert np.array_equal(out_c.cpu().numpy(), wants_b[0])
    for o, w in zip(outs_b, wants_b):
        assert np.array_equal(o.cpu().numpy(), w)


def test_freed_blocks_serve_other_streams_after_the_free(cuda):
    import torch

    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    es = 8
    probs = [([4, 2, 2, 4, 4, 3, 2, 2, 3, 2, 2], [10, 7, 1, 6, 3, 0, 4, 8, 9, 5, 2]),
             ([2, 4, 2, 2, 2, 4, 3, 2, 3, 2], [0, 6, 2, 4, 7, 5, 3, 8, 9, 1]),
             ([2, 2, 2, 4, 2, 3, 4, 2, 2, 3, 2], [9, 3, 2, 8, 7, 1, 10, 4, 5, 0, 6])]
    data = [_problem(d, p, es, 20 + k) for k, (d, p) in enumerate(probs)]
    for rnd in range(3):
        for k, (d, p) in enumerate(probs):
            s = s1 if (rnd + k) % 2 == 0 else s2
            h, w = data[k]
            inp = torch.from_numpy(h).cuda()
            out = torch.zeros_like(inp)
            torch.cuda.synchronize()
            with torch.cuda.stream(s):
                pl = _plan(d, p, es, s)
                pl.execute(inp.data_ptr(), out.data_ptr())
                pl.destroy()
            s.synchronize()
            assert np.array_equal(out.cpu().numpy(), w)


def test_small_tiles_hold_no_tables(cuda):
    """A plan whose tile has at most 6 ranks allocates nothing from the
    table arena and writes no tables; its first execute is correct."""
    import torch

    dims, perm, es = [512, 384, 96], [2, 0, 1], 4
    host, want = _problem_no_tables(dims, perm, es)
    inp = torch.from_numpy(host).cuda()
    out = torch.zeros_like(inp)
    s = torch.cuda.current_stream()
    before = L.table_arena_stats()
    with L.Plan(dims, perm, es, s) as pl:
        assert pl.info()["table_bytes"] == 0
        assert L.table_arena_stats() == before
        pl.execute(inp.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want)


def _problem_no_tables(dims, perm, es):
    assert L.describe(dims, perm, es)["table_bytes"] == 0
    host = np.random.default_rng(3).integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
    return host, O.transpose_np(host, dims, perm, es).view(np.uint8)
