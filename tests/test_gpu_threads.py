"""Plan, execute and destroy from several host threads at once.

LibreTT lets any thread call the API; here eight threads, each on its own
stream, repeatedly plan a random problem (plan cache on, learned selector),
execute it, check every output element on the device (librett_c_verify)
and destroy the plan.  This exercises the plan table, the plan cache, the
selector's per-thread buffers and the plan-table arena under contention.
(ctypes releases the interpreter lock during library calls, so the threads
run in the library concurrently.)
"""
import threading

import numpy as np
import pytest

import librett_gb300 as L
from tests import shapes as S

pytestmark = pytest.mark.gpu


def test_concurrent_plan_execute_destroy(cuda):
    import torch

    lib = L._lib.load()
    prev_cache = lib.librett_c_set_plan_cache(64)
    failures, errors = [], []

    def worker(tid):
        try:
            stream = torch.cuda.Stream()
            rng = np.random.default_rng(1000 + tid)
            g = torch.Generator(device="cuda")
            g.manual_seed(tid)
            with torch.cuda.stream(stream):
                for _ in range(40):
                    dims, perm, es = S.random_problem(rng, max_rank=6, max_vol=1 << 16)
                    nbytes = int(np.prod(dims)) * es
                    words = (nbytes + 7) // 8
                    inp = torch.randint(-(2 ** 62), 2 ** 62, (words,), device="cuda",
                                        dtype=torch.int64, generator=g)
                    out = torch.zeros_like(inp)
                    plan = L.Plan(dims, perm, es, stream)
                    plan.execute(inp.data_ptr(), out.data_ptr())
                    bad, first = L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), stream)
                    plan.destroy()
                    if bad:
                        failures.append((dims, perm, es, bad, first))
        except Exception as exc:  # reported below, in the main thread
            errors.append(repr(exc))

    try:
        threads = [threading.Thread(target=worker, args=(t,)) for t in range(8)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    finally:
        lib.librett_c_set_plan_cache(prev_cache)
    assert not errors, errors[:3]
    assert not failures, failures[:3]
