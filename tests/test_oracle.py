"""The oracle itself, pinned against LibreTT's known-answer checks (CPU only)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from tests import shapes as S
from tests.golden.make_golden import make_input

GOLDEN = Path(__file__).resolve().parent / "golden"
ROWS = json.loads((GOLDEN / "golden.json").read_text())
# The CPU run checks the fixtures up to 32 MB; the GPU tests check them all.
ROWS = [r for r in ROWS if r["nbytes"] <= 1 << 25]


@pytest.mark.parametrize("row", ROWS, ids=lambda r: f"{r['dims']}-{r['perm']}-{r['es']}-{r['input']}")
def test_oracle_matches_golden(row):
    dims, perm, es = row["dims"], row["perm"], row["es"]
    vol = int(np.prod(dims))
    inp = make_input(vol, es, row["input"])
    for out in (O.transpose_np(inp, dims, perm, es), O.transpose_c(inp, dims, perm, es, 4)):
        b = np.ascontiguousarray(out).view(np.uint8)
        assert b.nbytes == row["nbytes"]
        assert hashlib.sha256(b.tobytes()).hexdigest() == row["sha256"]


@pytest.mark.parametrize("es", [4, 8, 16])
def test_oracle_example_fixture(es):
    dims, perm = S.EXAMPLE
    want = np.load(GOLDEN / f"example_{es}.npy")
    inp = make_input(int(np.prod(dims)), es, "value")
    got = O.transpose_c(inp, dims, perm, es).view(np.uint8)
    assert np.array_equal(got, want)
    assert O.example_check(inp, got, dims, perm, es)


def test_restatements_agree_random():
    rng = np.random.default_rng(1)
    for _ in range(300):
        dims, perm, es = S.random_problem(rng, max_rank=8, max_vol=1 << 12)
        vol = int(np.prod(dims))
        inp = rng.integers(0, 256, vol * es, dtype=np.uint8)
        a = O.transpose_np(inp, dims, perm, es).view(np.uint8)
        b = O.transpose_c(inp, dims, perm, es, int(rng.integers(1, 9))).view(np.uint8)
        assert np.array_equal(a, b), (dims, perm, es)
        assert O.example_check(inp, a, dims, perm, es)
        p = O.fill_pattern(vol * es)
        assert O.pattern_check(O.transpose_c(p, dims, perm, es), dims, perm, es) is None


def test_pattern_check_catches_planted_mistakes():
    dims, perm, es = [4, 5, 6], [2, 0, 1], 8
    out = O.transpose_c(O.fill_pattern(120 * es), dims, perm, es).view(np.uint8).copy()
    assert O.pattern_check(out, dims, perm, es) is None
    out[8 * 17] ^= 0x10  # corrupt element 17
    bad = O.pattern_check(out, dims, perm, es)
    assert bad is not None and bad[0] == 17
    swapped = O.transpose_c(O.fill_pattern(120 * es), dims, [2, 1, 0], es)
    assert O.pattern_check(swapped, dims, perm, es) is not None


def test_thread_count_invariance():
    rng = np.random.default_rng(5)
    dims, perm, es = [37, 11, 23, 5], [3, 1, 0, 2], 16
    inp = rng.integers(0, 256, int(np.prod(dims)) * es, dtype=np.uint8)
    ref = O.transpose_c(inp, dims, perm, es, 1).view(np.uint8)
    for t in (2, 3, 7, 16):
        assert np.array_equal(O.transpose_c(inp, dims, perm, es, t).view(np.uint8), ref)


RANDOM = GOLDEN / "librett_random.json"
RANDOM_CASES = ([c for c in json.loads(RANDOM.read_text())["cases"] if c["bytes"] <= 1 << 25]
                if RANDOM.exists() else [])


@pytest.mark.parametrize("case", RANDOM_CASES, ids=[c["name"] for c in RANDOM_CASES])
def test_oracle_matches_librett_random(case):
    """The oracle's output digests like LibreTT's own output on the seeded
    random-bit inputs (the cases up to 32 MB; the GPU tests check them all
    against the engine)."""
    from oracle import vectors as V

    dims, perm, es = case["dims"], case["perm"], case["es"]
    inp = V.input_bytes(case["key"], case["bytes"])
    out = O.transpose_c(inp, dims, perm, es, 4)
    assert V.tree_digest(np.ascontiguousarray(out).view(np.uint8)) == case["digest"]


def test_random_inputs_restatements_agree():
    """oracle/vectors.py's numpy and torch generators give the same bytes,
    and the first words for key 0 are SplitMix64's published sequence."""
    import torch

    from oracle import vectors as V

    assert [int(x) for x in V.words_np(0, 0, 2)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4]
    for key, n in ((0x6C69627265747400, 4099), (12345, 40), (2 ** 64 - 1, 17)):
        t = torch.empty(n, dtype=torch.uint8)
        V.fill_torch(t, key, chunk_words=64)
        assert np.array_equal(t.numpy(), V.input_bytes(key, n))
