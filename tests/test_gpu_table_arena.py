"""Plan tables come from a host-side arena with stream-ordered reuse.

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


def _problem(dims, perm, es, seed):
    host = np.random.default_rng(seed).integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
    return host, O.transpose_np(host, dims, perm, es).view(np.uint8)


def test_reuse_waits_for_the_freeing_stream(cuda):
    import torch

    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    es = 4
    dims_a, perm_a = [512, 384, 96], [2, 0, 1]
    host_a, want_a = _problem(dims_a, perm_a, es, 1)
    inp_a = torch.from_numpy(host_a).cuda()
    outs_a = [torch.zeros_like(inp_a) for _ in range(4)]
    # other problems, other tables, the same range of table sizes
    others = [([384, 512, 96], [1, 2, 0]), ([96, 512, 384], [2, 1, 0]), ([512, 96, 384], [1, 0, 2]),
              ([300, 200, 250], [2, 0, 1]), ([250, 300, 200], [1, 2, 0]), ([64, 64, 64, 64], [3, 1, 0, 2])]
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
        plan_a = L.Plan(dims_a, perm_a, es, s1)
        for k in range(16):
            plan_a.execute(inp_a.data_ptr(), outs_a[k % 4].data_ptr())
        plan_a.destroy()  # its transposes are still queued behind the copies
        # the same stream may reuse the block at once
        plan_c = L.Plan(others[0][0], others[0][1], es, s1)
        out_c = torch.zeros_like(ins_b[0])
        plan_c.execute(ins_b[0].data_ptr(), out_c.data_ptr())
    assert s1.query() is False, "the first stream finished too early for this test to mean anything"
    plans_b = []
    for k, (d, p) in enumerate(others):
        pb = L.Plan(d, p, es, s2)
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
    probs = [([96, 80, 70], [2, 0, 1]), ([70, 96, 80], [1, 2, 0]), ([80, 70, 96], [2, 1, 0])]
    data = [_problem(d, p, es, 20 + k) for k, (d, p) in enumerate(probs)]
    for rnd in range(3):
        for k, (d, p) in enumerate(probs):
            s = s1 if (rnd + k) % 2 == 0 else s2
            h, w = data[k]
            inp = torch.from_numpy(h).cuda()
            out = torch.zeros_like(inp)
            torch.cuda.synchronize()
            with torch.cuda.stream(s):
                pl = L.Plan(d, p, es, s)
                pl.execute(inp.data_ptr(), out.data_ptr())
                pl.destroy()
            s.synchronize()
            assert np.array_equal(out.cpu().numpy(), w)
