"""Parity at the benchmarks' full sizes, through the device verifier.

The verifier (librett_c_verify, itself checked against the oracle with
planted mistakes in test_gpu_verify.py) compares every output element with
the input element the transpose formula names.  Here it checks
* the whole 10,000-transpose grouped batch of the grouped benchmark
  (30.3 GB in, 30.3 GB out), executed once as one group;
* the first suite problems of the default benchmark at their full size
  (1 GiB in, 1 GiB out each), planned by the default planner;
* volumes past 2^31 elements (LibreTT's 32-bit range; 8.6 and 17.2 GB each
  way) through the tile, copy and row-copy kernels, with a round trip through
  the inverse permutation as well.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

import librett_gb300 as L
from librett_gb300.workloads import grouped_problems, packed_offsets

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def _random_bytes(nbytes, seed):
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    words = (nbytes + 7) // 8
    return torch.randint(-(2 ** 62), 2 ** 62, (words,), device="cuda", dtype=torch.int64,
                         generator=g).view(torch.uint8)[:nbytes]


def test_grouped_batch_every_member(cuda):
    import torch

    problems = grouped_problems(10000)
    offs, total = packed_offsets(problems)
    inp = _random_bytes(total, 11)
    out = torch.zeros(total, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    base_in, base_out = inp.data_ptr(), out.data_ptr()
    plans = [L.Plan(d, p, es, s) for d, p, es in problems]
    try:
        with L.Group(plans, [base_in + o for o in offs], [base_out + o for o in offs], s) as g:
            g.execute()
            torch.cuda.synchronize()
        bad = []
        for (d, p, es), o in zip(problems, offs):
            n, first = L.verify(d, p, es, base_in + o, base_out + o, s)
            if n:
                bad.append((d, p, es, n, first))
        assert not bad, bad[:5]
    finally:
        for pl in plans:
            pl.destroy()
    del inp, out
    torch.cuda.empty_cache()


def test_suite_problems_full_size(cuda):
    import torch

    sys.path.insert(0, str(ROOT))
    import bench

    problems = bench.suite_problems(200)[:12]
    maxb = max(bench.problem_bytes(p) for p in problems)
    inp = _random_bytes(maxb, 12)
    out = torch.empty(maxb, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    methods = set()
    for d, p, es in problems:
        out.zero_()
        with L.Plan(d, p, es, s) as pl:
            methods.add(pl.info()["method"])
            pl.execute(inp.data_ptr(), out.data_ptr())
            n, first = L.verify(d, p, es, inp.data_ptr(), out.data_ptr(), s)
        assert n == 0, (d, p, es, n, first)
    assert len(methods) >= 3  # copies, tiles of several kinds
    del inp, out
    torch.cuda.empty_cache()


@pytest.mark.parametrize("dims, perm, es", [
    ([65539, 32769], [1, 0], 4),          # 2,147,647,491 elements, 8.6 GB each way
    ([3, 46341, 15461], [2, 0, 1], 8),    # 2,149,434,603 elements, 17.2 GB each way
    ([65539, 32769], [0, 1], 4),          # identity: one rank-1 copy
    ([64, 33555, 1001], [0, 2, 1], 4),    # leading rank kept: 2,149,667,520 elements
])
def test_beyond_2_31_elements(cuda, dims, perm, es):
    """Volumes past 2^31 elements (LibreTT's int32 range): every output element
    checked on the device, and the inverse permutation returns the input."""
    import torch

    vol = int(np.prod(dims))
    assert vol > 2 ** 31
    nbytes = vol * es
    inp = _random_bytes(nbytes, 13)
    out = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    with L.Plan(dims, perm, es, s) as p1:
        p1.execute(inp.data_ptr(), out.data_ptr())
        n, first = L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), s)
    assert n == 0, (n, first)
    back = torch.empty_like(inp)
    odims = [dims[p] for p in perm]
    inv = [0] * len(perm)
    for i, p in enumerate(perm):
        inv[p] = i
    with L.Plan(odims, inv, es, s) as p2:
        p2.execute(out.data_ptr(), back.data_ptr())
        torch.cuda.synchronize()
    assert torch.equal(back, inp)
    del inp, out, back
    torch.cuda.empty_cache()


def test_row_copy_beyond_2_31_elements(cuda):
    """The row-copy kernel (LibreTT's TiledCopy) past 2^31 elements: its
    candidate is the first one whenever the leading rank stays in place."""
    import torch

    dims, perm, es = [64, 33555, 1001], [0, 2, 1], 4
    vol = int(np.prod(dims))
    inp = _random_bytes(vol * es, 14)
    out = torch.empty(vol * es, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    with L.Plan(dims, perm, es, s, candidate=0) as p:
        assert L.METHOD_NAMES[p.info()["method"]] == "TiledCopy"
        p.execute(inp.data_ptr(), out.data_ptr())
        n, first = L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), s)
    assert n == 0, (n, first)
    del inp, out
    torch.cuda.empty_cache()
