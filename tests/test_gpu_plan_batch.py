"""librett_c_plan_batch: librettPlan on many problems in one call."""
import ctypes

import numpy as np
import pytest

import librett_gb300 as L
from librett_gb300 import _lib
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PROBS = [([64, 48, 32], [2, 0, 1], 4), ([300, 7, 11], [1, 2, 0], 8),
         ([4, 6, 128, 5, 16], [3, 0, 4, 2, 1], 16), ([1000], [0], 8),
         ([33, 65, 17], [1, 2, 0], 8), ([7, 1, 9], [2, 1, 0], 4)]


def test_plan_batch_matches_single_plans(cuda):
    import torch

    s = torch.cuda.current_stream()
    for sync in (False, True):
        plans, us = L.plan_batch(PROBS, s, synchronize=sync, timings=True)
        try:
            assert len(plans) == len(PROBS) and all(u > 0 for u in us)
            for pl, (d, p, es) in zip(plans, PROBS):
                with L.Plan(d, p, es, s) as one:
                    a, b = pl.info(), one.info()
                    assert (a["method"], a["tile_extent"], a["pipeline"], a["candidate"]) == \
                           (b["method"], b["tile_extent"], b["pipeline"], b["candidate"])
                host = np.random.default_rng(1).integers(0, 256, int(np.prod(d)) * es,
                                                         dtype=np.uint8)
                inp = torch.from_numpy(host).cuda()
                out = torch.zeros_like(inp)
                pl.execute(inp.data_ptr(), out.data_ptr())
                torch.cuda.synchronize()
                assert np.array_equal(out.cpu().numpy(), O.transpose_np(host, d, p, es).view(np.uint8))
        finally:
            for pl in plans:
                pl.destroy()


def test_plan_batch_error_releases_earlier_plans(cuda):
    import torch

    s = torch.cuda.current_stream()
    bad = PROBS[:2] + [([4, 4], [0, 0], 8)] + PROBS[2:]  # not a permutation
    lib = _lib.load()
    n = len(bad)
    ranks = (ctypes.c_int * n)(*[len(d) for d, _, _ in bad])
    dims = (ctypes.c_int * sum(len(d) for d, _, _ in bad))(*[x for d, _, _ in bad for x in d])
    perms = (ctypes.c_int * sum(len(d) for d, _, _ in bad))(*[x for _, p, _ in bad for x in p])
    sizes = (ctypes.c_size_t * n)(*[es for _, _, es in bad])
    hs = (ctypes.c_uint * n)()
    rc = lib.librett_c_plan_batch(n, ranks, dims, perms, sizes, ctypes.c_void_p(s.cuda_stream),
                                  0, hs, None)
    assert rc == L.LIBRETT_INVALID_PARAMETER
    info = L.PlanInfo()
    for h in hs[:2]:  # the plans made before the failing problem were destroyed
        assert lib.librett_c_plan_info(h, ctypes.byref(info)) == L.LIBRETT_INVALID_PLAN
