"""CUDA-error paths, driven by host-side fault injection.

LibreTT exits the process on any CUDA error (src/GpuUtils.h:47-56).  This
library returns LIBRETT_INTERNAL_ERROR instead and must stay usable.  The
failures here are made on the host (librett_c_inject_fault reports a CUDA
error before the device is called), so no GPU ever faults: each test arms one
site, checks the error code, then checks that the next call through the same
path succeeds and transposes correctly.

The bulk-copy pipeline's bounded mbarrier wait is driven the same way: a
test launch arms more bytes than the copies deliver (a count nothing
completes), so the wait runs out and the kernel reports it in the plan's
status word; the copies themselves land normally.
"""
import ctypes
import time

import numpy as np
import pytest

import librett_gb300 as L
from librett_gb300 import _lib
from oracle import oracle as O

DIMS, PERM, ES = [37, 8, 19, 6], [2, 0, 3, 1], 8  # a tile plan (addresses computed in the kernel)
# candidates with tiles of more than 6 ranks: their plans allocate and write
# offset tables
TDIMS, TPERM, TES = [4, 2, 2, 4, 4, 3, 2, 2, 3, 2, 2], [10, 7, 1, 6, 3, 0, 4, 8, 9, 5, 2], 8


def _data(dims, es, seed=3):
    import torch

    host = np.random.default_rng(seed).integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
    return host, torch.from_numpy(host).cuda()


@pytest.fixture
def disarm():
    yield
    for site in (L.FAULT_TABLE_ALLOC, L.FAULT_GROUP_ALLOC, L.FAULT_LAUNCH):
        L.inject_fault(site, -1)


def test_fault_sites_are_validated():
    lib = _lib.load()
    assert lib.librett_c_inject_fault(3, 0) == L.LIBRETT_INVALID_PARAMETER
    assert lib.librett_c_inject_fault(-1, 0) == L.LIBRETT_INVALID_PARAMETER
    for site in (0, 1, 2):
        assert lib.librett_c_inject_fault(site, -1) == L.LIBRETT_SUCCESS


@pytest.mark.gpu
def test_plan_table_allocation_failure(cuda, disarm):
    import torch

    host, inp = _data(TDIMS, TES)
    out = torch.zeros_like(inp)
    s = torch.cuda.current_stream()
    lib = _lib.load()
    prev = lib.librett_c_set_plan_cache(0)
    try:
        n = L.describe(TDIMS, TPERM, TES)["num_candidates"]
        tc = next(c for c in range(n)
                  if L.describe(TDIMS, TPERM, TES, candidate=c)["table_bytes"] > 0)
        L.inject_fault(L.FAULT_TABLE_ALLOC, 0)
        with pytest.raises(L.LibrettError) as e:
            L.Plan(TDIMS, TPERM, TES, s, candidate=tc)
        assert e.value.code == L.LIBRETT_INTERNAL_ERROR
        L.inject_fault(L.FAULT_TABLE_ALLOC, 0)
        with pytest.raises(L.LibrettError) as e:
            L.Plan(TDIMS, TPERM, TES, s, measure=(inp.data_ptr(), out.data_ptr()))
        assert e.value.code == L.LIBRETT_INTERNAL_ERROR
        # disarmed after firing: the same calls now succeed
        with L.Plan(TDIMS, TPERM, TES, s, candidate=tc) as p:
            assert p.info()["table_bytes"] > 0
            p.execute(inp.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(),
                              O.transpose_np(host, TDIMS, TPERM, TES).view(np.uint8))
    finally:
        lib.librett_c_set_plan_cache(prev)


@pytest.mark.gpu
def test_execute_launch_failure(cuda, disarm):
    import torch

    host, inp = _data(DIMS, ES)
    out = torch.zeros_like(inp)
    s = torch.cuda.current_stream()
    want = O.transpose_np(host, DIMS, PERM, ES).view(np.uint8)
    with L.Plan(DIMS, PERM, ES, s) as p:
        L.inject_fault(L.FAULT_LAUNCH, 1)  # the first execute passes, the second fails
        p.execute(inp.data_ptr(), out.data_ptr())
        with pytest.raises(L.LibrettError) as e:
            p.execute(inp.data_ptr(), out.data_ptr())
        assert e.value.code == L.LIBRETT_INTERNAL_ERROR
        out.zero_()
        p.execute(inp.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want)


@pytest.mark.gpu
def test_group_failures(cuda, disarm):
    import torch

    probs = [(DIMS, PERM, ES), ([33, 17], [1, 0], 4), ([5, 7, 9, 3], [3, 1, 0, 2], 16)]
    nbytes = [int(np.prod(d)) * e for d, _, e in probs]
    offs = np.concatenate([[0], np.cumsum([(n + 255) // 256 * 256 for n in nbytes])])
    host = np.random.default_rng(5).integers(0, 256, int(offs[-1]), dtype=np.uint8)
    gin = torch.from_numpy(host).cuda()
    gout = torch.zeros_like(gin)
    s = torch.cuda.current_stream()
    ins = [gin.data_ptr() + int(o) for o in offs[:-1]]
    outs = [gout.data_ptr() + int(o) for o in offs[:-1]]
    plans = [L.Plan(d, p, e, s) for d, p, e in probs]
    try:
        L.inject_fault(L.FAULT_GROUP_ALLOC, 0)
        with pytest.raises(L.LibrettError) as e:
            L.Group(plans, ins, outs, s)
        assert e.value.code == L.LIBRETT_INTERNAL_ERROR
        with L.Group(plans, ins, outs, s) as g:
            L.inject_fault(L.FAULT_LAUNCH, 0)
            with pytest.raises(L.LibrettError) as e:
                g.execute()
            assert e.value.code == L.LIBRETT_INTERNAL_ERROR
            g.execute()
            torch.cuda.synchronize()
        res = gout.cpu().numpy()
        for (d, p, e), o, n in zip(probs, offs, nbytes):
            assert np.array_equal(res[o:o + n], O.transpose_np(host[o:o + n], d, p, e).view(np.uint8))
    finally:
        for p in plans:
            p.destroy()


@pytest.mark.gpu
def test_noalloc_launch_failure(cuda, disarm):
    import torch

    host, inp = _data(DIMS, ES)
    out = torch.zeros_like(inp)
    s = torch.cuda.current_stream()
    L.inject_fault(L.FAULT_LAUNCH, 0)
    assert L.transpose_noalloc(DIMS, PERM, ES, s, inp.data_ptr(),
                               out.data_ptr()) == L.LIBRETT_INTERNAL_ERROR
    assert L.transpose_noalloc(DIMS, PERM, ES, s, inp.data_ptr(),
                               out.data_ptr()) == L.LIBRETT_SUCCESS
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), O.transpose_np(host, DIMS, PERM, ES).view(np.uint8))


def _bulk_candidate(dims, perm, es):
    n = L.describe(dims, perm, es)["num_candidates"]
    for c in range(n):
        info = L.describe(dims, perm, es, candidate=c)
        if info["pipeline"] == 3 and info["num_tiles"] <= 4:
            return c, info
    raise AssertionError("no bulk-copy candidate with at most 4 tiles")


def test_bulk_wait_test_arguments():
    lib = _lib.load()
    st = ctypes.c_uint(0)
    assert lib.librett_c_bulk_wait_test(0, None, None, 16, ctypes.byref(st)) != L.LIBRETT_SUCCESS
    assert lib.librett_c_bulk_wait_test(0, None, None, 16, None) == L.LIBRETT_INVALID_PARAMETER


@pytest.mark.gpu
def test_bulk_wait_runs_out_and_reports(cuda):
    """Each CTA of a bulk-copy launch whose mbarrier never completes gives up
    after its time limit (about 1 s, then at most 1 s more for its copies),
    sets status bit 0 and stores nothing; the plan's status reads 0 again
    afterwards and its next execute is correct."""
    import torch

    dims, perm, es = [64, 32], [1, 0], 8
    cand, info = _bulk_candidate(dims, perm, es)
    host, inp = _data(dims, es)
    out = torch.full_like(inp, 0xA5)
    s = torch.cuda.current_stream()
    lib = _lib.load()
    want = O.transpose_np(host, dims, perm, es).view(np.uint8)
    with L.Plan(dims, perm, es, s, candidate=cand) as p:
        assert p.info()["pipeline"] == 3
        # wrong plan kind or arguments are refused before any launch
        st = ctypes.c_uint(7)
        for extra in (0, 4097):
            assert lib.librett_c_bulk_wait_test(p.handle, inp.data_ptr(), out.data_ptr(), extra,
                                                ctypes.byref(st)) == L.LIBRETT_INVALID_PARAMETER
        assert lib.librett_c_bulk_wait_test(p.handle, inp.data_ptr() + 8, out.data_ptr(), 16,
                                            ctypes.byref(st)) == L.LIBRETT_INVALID_PARAMETER
        torch.cuda.synchronize()
        t0 = time.monotonic()
        rc = lib.librett_c_bulk_wait_test(p.handle, inp.data_ptr(), out.data_ptr(), 16,
                                          ctypes.byref(st))
        waited = time.monotonic() - t0
        assert rc == L.LIBRETT_SUCCESS and st.value == 1
        assert 0.9 < waited < 30.0, waited
        assert bool((out == 0xA5).all())  # no CTA stored
        assert p.status() == 0
        p.execute(inp.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        assert p.status() == 0
    assert np.array_equal(out.cpu().numpy(), want)
    with L.Plan(dims, perm, es, s) as p:  # a plan that is not bulk-copy is refused
        if p.info()["pipeline"] != 3:
            assert lib.librett_c_bulk_wait_test(p.handle, inp.data_ptr(), out.data_ptr(), 16,
                                                ctypes.byref(st)) == L.LIBRETT_INVALID_PARAMETER
