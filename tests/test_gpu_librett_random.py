"""Parity with LibreTT's own CUDA build at the benchmark configurations.

tests/golden/librett_random.json holds, for C1, C3a (4 GB), C3b, the first
40 problems of the random-shape suite (1 GiB each) and the first 20 problems
of the batched distribution, the digest of the output LibreTT's unmodified
build produced on a GB300 for a seeded random-bit input
(oracle/ref_bench/run_ref.py --random --write-fixture).  Here the engine
transposes the same inputs through the C-ABI and its outputs must digest
identically: bit-exact agreement with LibreTT on the shapes the benchmark
times, not only on the small known-answer cases.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import librett_gb300 as L
from oracle import vectors as V

pytestmark = pytest.mark.gpu

FIXTURE = Path(__file__).resolve().parent / "golden" / "librett_random.json"
CASES = json.loads(FIXTURE.read_text())["cases"] if FIXTURE.exists() else []


def _digest_device(buf) -> str:
    return V.tree_digest(buf.cpu().numpy())


def test_fixture_covers_the_benchmark_configurations():
    assert FIXTURE.exists(), "run oracle/ref_bench/run_ref.py --random --write-fixture"
    names = [c["name"] for c in CASES]
    assert names[:3] == ["c1", "c3a", "c3b"]
    assert sum(n.startswith("suite") for n in names) == 40
    assert sum(n.startswith("grouped") for n in names) == 20


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_plan_execute_matches_librett(cuda, case):
    import torch

    dims, perm, es = case["dims"], case["perm"], case["es"]
    nbytes = int(np.prod(dims)) * es
    assert nbytes == case["bytes"]
    inp = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    V.fill_torch(inp, case["key"])
    out = torch.full((nbytes,), 0xA5, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    with L.Plan(dims, perm, es, stream) as plan:
        plan.execute(inp.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    assert _digest_device(out) == case["digest"], (case["name"], dims, perm, es)


def test_grouped_matches_librett(cuda):
    """The batched problems once more, as one grouped execution."""
    import torch

    cases = [c for c in CASES if c["name"].startswith("grouped")]
    offs, total = [], 0
    for c in cases:
        offs.append(total)
        total += (c["bytes"] + 255) // 256 * 256
    inp = torch.empty(total, dtype=torch.uint8, device="cuda")
    for c, o in zip(cases, offs):
        V.fill_torch(inp[o:o + c["bytes"]], c["key"])
    out = torch.full((total,), 0xA5, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    plans = [L.Plan(c["dims"], c["perm"], c["es"], stream) for c in cases]
    try:
        with L.Group(plans, [inp.data_ptr() + o for o in offs],
                     [out.data_ptr() + o for o in offs], stream) as g:
            g.execute()
            torch.cuda.synchronize()
    finally:
        for p in plans:
            p.destroy()
    host = out.cpu().numpy()
    for c, o in zip(cases, offs):
        assert V.tree_digest(host[o:o + c["bytes"]]) == c["digest"], c["name"]
