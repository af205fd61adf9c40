"""The plan cache: a repeated shape reuses the planner's choice.

A second librettPlan of the same fused problem on the same device must be a
cache hit, produce the same plan description and the same bit-exact output;
shapes that fuse to the same problem share an entry; capacity 0 disables the
cache; changing the selector clears it.
"""
import ctypes

import numpy as np
import pytest

import librett_gb300 as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _stats():
    h, m, n = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    L._lib.load().librett_c_plan_cache_stats(ctypes.byref(h), ctypes.byref(m), ctypes.byref(n))
    return h.value, m.value, n.value


def _run(dims, perm, es, host, stream):
    import torch

    inp = torch.from_numpy(host).cuda()
    out = torch.zeros_like(inp)
    with L.Plan(dims, perm, es, stream) as p:
        info = p.info()
        p.execute(inp.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy(), info


def test_repeat_is_a_hit(cuda):
    import torch

    lib = L._lib.load()
    prev = lib.librett_c_set_plan_cache(64)
    try:
        stream = torch.cuda.current_stream()
        dims, perm, es = [37, 5, 41, 3], [2, 0, 3, 1], 8
        host = np.random.default_rng(1).integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
        want = O.transpose_np(host, dims, perm, es).view(np.uint8)
        h0, m0, _ = _stats()
        got1, info1 = _run(dims, perm, es, host, stream)
        h1, m1, _ = _stats()
        got2, info2 = _run(dims, perm, es, host, stream)
        h2, m2, _ = _stats()
        assert (h1 - h0, m1 - m0) == (0, 1) or (h1 - h0, m1 - m0) == (1, 0)
        assert (h2 - h1, m2 - m1) == (1, 0)
        assert info1 == info2
        assert np.array_equal(got1, want) and np.array_equal(got2, want)
        # unit dims fuse away: the same fused problem, the same entry
        got3, _ = _run([37, 1, 5, 41, 1, 3], [3, 0, 4, 5, 1, 2], es, host, stream)
        h3, _, _ = _stats()
        assert h3 - h2 == 1
        assert np.array_equal(got3, O.transpose_np(host, [37, 1, 5, 41, 1, 3], [3, 0, 4, 5, 1, 2],
                                                   es).view(np.uint8))
    finally:
        lib.librett_c_set_plan_cache(prev)


def test_capacity_zero_and_clear(cuda):
    import torch

    lib = L._lib.load()
    prev = lib.librett_c_set_plan_cache(0)
    try:
        stream = torch.cuda.current_stream()
        dims, perm, es = [12, 34, 56], [1, 2, 0], 4
        host = np.random.default_rng(2).integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
        h0, m0, n0 = _stats()
        _run(dims, perm, es, host, stream)
        _run(dims, perm, es, host, stream)
        h1, m1, n1 = _stats()
        assert (h1, m1, n1) == (h0, m0, 0)
        lib.librett_c_set_plan_cache(16)
        _run(dims, perm, es, host, stream)
        assert _stats()[2] == 1
        old = lib.librett_c_set_plan_selector(1)   # clears the cache
        assert _stats()[2] == 0
        lib.librett_c_set_plan_selector(old)
    finally:
        lib.librett_c_set_plan_cache(prev)
