"""Parity of the CUDA path with the CPU oracle, through the C-ABI.

Every comparison is bit-exact (the engine moves raw words).  Buffers carry
64-byte guard bands filled with a canary that must survive each launch.
Shapes follow LibreTT's own tests (tests/librett_test.cpp test1/test3,
tests/example.cpp) plus seeded random problems and the full-size
small-leading-dimension stress shapes, which are checked through
size-independent properties (round trip, sampled gather formula).
"""
import ctypes

import numpy as np
import pytest

import librett_gb300 as L
from oracle import oracle as O
from tests import shapes as S

pytestmark = pytest.mark.gpu

GUARD = 64
CANARY = 0xA5


def _run(dims, perm, es, host_bytes, *, candidate=None, measure=False, stream=None, offset=0):
    import torch

    dev = torch.device("cuda:0")
    n = host_bytes.nbytes
    inp = torch.zeros(n + 2 * GUARD, dtype=torch.uint8, device=dev)
    out = torch.full((n + 2 * GUARD,), CANARY, dtype=torch.uint8, device=dev)
    inp[GUARD + offset:GUARD + offset + n].copy_(torch.from_numpy(np.ascontiguousarray(host_bytes)))
    ip = inp.data_ptr() + GUARD + offset
    op = out.data_ptr() + GUARD + offset
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    plan = L.Plan(dims, perm, es, s, measure=(ip, op) if measure else None, candidate=candidate)
    try:
        plan.execute(ip, op)
        torch.cuda.synchronize(dev)
        info = plan.info()
        info["status"] = plan.status()
    finally:
        plan.destroy()
    res = out.cpu().numpy()
    lo, hi = GUARD + offset, GUARD + offset + n
    assert (res[:lo] == CANARY).all(), "write before the output buffer"
    assert (res[hi:] == CANARY).all(), "write after the output buffer"
    return res[lo:hi], info


def _check(dims, perm, es, rng=None, **kw):
    vol = int(np.prod(dims))
    if rng is None:
        host = O.fill_pattern(vol * es)
    else:
        host = rng.integers(0, 256, vol * es, dtype=np.uint8)
    got, info = _run(dims, perm, es, host, **kw)
    want = O.transpose_np(host, dims, perm, es).view(np.uint8)
    if not np.array_equal(got, want):
        bad = int(np.nonzero(got != want)[0][0])
        raise AssertionError(f"dims {dims} perm {perm} es {es} info {info}: first bad byte {bad}")
    return info


def test_c1_plain_small(cuda):
    dims, perm, es = S.C1
    vol = int(np.prod(dims))
    host = O.fill_pattern(vol * es)
    got, _ = _run(dims, perm, es, host)
    assert np.array_equal(got, O.transpose_c(host, dims, perm, es).view(np.uint8))
    assert O.pattern_check(got, dims, perm, es) is None


@pytest.mark.parametrize("es", [4, 8, 16])
def test_example_shape(cuda, es):
    dims, perm = S.EXAMPLE
    vol = int(np.prod(dims))
    host = O.fill_pattern(vol * es)
    got, _ = _run(dims, perm, es, host)
    assert O.example_check(host, got, dims, perm, es)
    assert O.pattern_check(got, dims, perm, es) is None


@pytest.mark.parametrize("rank", [2, 3, 4, 5, 6, 7])
def test_all_permutations(cuda, rank):
    cap = {6: 120, 7: 60}.get(rank)
    for dims, perm in S.test1_cases(max_rank=rank, max_perms_per_rank=cap, seed=rank):
        if len(dims) != rank:
            continue
        for es in (4, 8, 16):
            _check(dims, perm, es)


@pytest.mark.parametrize("case", range(len(S.TEST3)))
@pytest.mark.parametrize("es", [4, 8, 16])
def test_handpicked_shapes(cuda, case, es):
    dims, perm = S.TEST3[case]
    _check(dims, perm, es)


def test_random_problems(cuda):
    rng = np.random.default_rng(20261203)
    for _ in range(250):
        dims, perm, es = S.random_problem(rng, max_rank=8, max_vol=1 << 18)
        _check(dims, perm, es, rng=rng)


def test_unit_dims_and_degenerate(cuda):
    cases = [([1], [0]), ([1, 1, 1], [2, 0, 1]), ([7], [0]), ([1, 5, 1, 3], [3, 2, 1, 0]),
             ([2, 1, 3], [1, 2, 0]), ([1000, 1], [1, 0]), ([3, 5], [0, 1])]
    for dims, perm in cases:
        for es in (4, 8, 16):
            _check(dims, perm, es)


def test_every_candidate(cuda):
    rng = np.random.default_rng(7)
    probs = [([64, 48, 32], [2, 0, 1], 4), ([4, 6, 128, 5, 16], [3, 0, 4, 2, 1], 16),
             ([2, 3, 4, 5, 512, 16], [5, 3, 1, 4, 0, 2], 4), ([300, 7, 11], [0, 2, 1], 8),
             ([33, 65, 17], [1, 2, 0], 8), ([1024, 1024], [1, 0], 4),
             # element loads with 16-byte stores and an odd unit count
             ([51, 2, 1354, 2, 9], [1, 3, 0, 2, 4], 4),
             # bulk-copy tiles above 48 KB of shared memory (opt-in limit)
             ([128, 64, 6], [1, 0, 2], 16), ([96, 100, 24], [1, 0, 2], 16)]
    big_bulk = 0
    for dims, perm, es in probs:
        n = L.describe(dims, perm, es)["num_candidates"]
        assert n >= 1
        for c in range(n):
            info = _check(dims, perm, es, rng=rng, candidate=c)
            assert info["status"] == 0
            big_bulk += info["pipeline"] == 3 and info["smem_bytes"] > 48 * 1024
    assert big_bulk >= 2


# (dims, perm, es, candidate) of flat (pipeline 2) and bulk-copy (3) tiles
# of 1..7 tile ranks, with store units that cross the first output tile rank
# and without: tiles of up to 6 ranks address their units arithmetically,
# larger ones read offset tables
ADDRESSING_CASES = [
    ([10, 10, 8], [0, 2, 1], 8, 6), ([6, 9, 8, 3, 3, 6], [0, 1, 4, 3, 5, 2], 16, 10),
    ([11, 11, 4, 8, 8, 4], [5, 0, 4, 2, 1, 3], 8, 8), ([8, 9, 4], [1, 0, 2], 4, 2),
    ([2, 9, 8], [1, 2, 0], 4, 1), ([8, 9, 4], [1, 0, 2], 4, 3),
    ([2, 3, 6, 5, 10, 7], [2, 4, 1, 3, 5, 0], 16, 11), ([9, 6, 2, 4, 9], [0, 3, 4, 2, 1], 4, 4),
    ([10, 10, 8], [0, 2, 1], 8, 1), ([8, 9, 4], [1, 0, 2], 4, 1),
    ([2, 3, 6, 5, 10, 7], [2, 4, 1, 3, 5, 0], 16, 2),
    ([3, 4, 3, 10, 10, 7, 2], [5, 6, 1, 4, 2, 3, 0], 4, 4),
    ([2, 3, 6, 5, 10, 7], [2, 4, 1, 3, 5, 0], 16, 3),
    ([3, 4, 3, 10, 10, 7, 2], [5, 6, 1, 4, 2, 3, 0], 4, 5),
    ([2, 3, 6, 5, 10, 7], [2, 4, 1, 3, 5, 0], 16, 0),
    ([3, 4, 3, 10, 10, 7, 2], [5, 6, 1, 4, 2, 3, 0], 4, 0),
    ([2, 3, 6, 5, 10, 7], [2, 4, 1, 3, 5, 0], 16, 1),
    ([3, 4, 3, 10, 10, 7, 2], [5, 6, 1, 4, 2, 3, 0], 4, 1),
    ([2, 3, 6, 5, 10, 7], [2, 4, 1, 3, 5, 0], 16, 10),
    ([7, 5, 2, 2, 4, 3, 9, 4], [5, 0, 2, 3, 7, 6, 1, 4], 4, 0),
    ([8, 5, 8, 2, 5, 3, 5, 3], [6, 1, 3, 5, 0, 7, 4, 2], 4, 1),
    ([7, 5, 2, 2, 4, 3, 9, 4], [5, 0, 2, 3, 7, 6, 1, 4], 4, 1),
    ([6, 2, 3, 2, 4, 7, 4], [4, 0, 3, 5, 2, 6, 1], 4, 0),
    ([2, 4, 3, 2, 5, 8, 8], [4, 1, 6, 2, 0, 5, 3], 8, 6),
    ([6, 2, 3, 2, 4, 7, 4], [4, 0, 3, 5, 2, 6, 1], 4, 1),
    ([2, 4, 3, 2, 5, 8, 8], [4, 1, 6, 2, 0, 5, 3], 8, 7),
]


def _addressing_key(info, es):
    ext, fp, r = info["tile_extent"], info["fused_perm"], info["fused_rank"]
    ntr = sum(1 for e in ext[:r] if e > 1)
    first_out = next(q for q in fp[:r] if ext[q] > 1)
    sv = info["unit_out_bytes"] // es
    return min(ntr, 7), info["pipeline"], sv > 1 and ext[first_out] % sv != 0


def test_addressing_every_rank_count(cuda):
    """Flat and bulk-copy tiles of every rank count, with and without store
    units that cross the first output tile rank, bit-exact; tables exist
    exactly for tiles of more than 6 ranks."""
    rng = np.random.default_rng(13)
    keys = set()
    for dims, perm, es, c in ADDRESSING_CASES:
        info = L.describe(dims, perm, es, candidate=c)
        key = _addressing_key(info, es)
        keys.add(key)
        assert (info["table_bytes"] > 0) == (key[0] >= 7), (dims, perm, es, c, info["table_bytes"])
        got = _check(dims, perm, es, rng=rng, candidate=c)
        assert got["status"] == 0
    assert keys == {(n, p, s) for n in range(1, 8) for p in (2, 3) for s in (False, True)} - {
        (1, 2, True), (1, 3, True)}, keys


def test_every_candidate_all_pipelines(cuda):
    """Candidate set 1: the persistent register-staged and cp.async
    pipelines and the bulk-copy pipeline (one cp.async.bulk per contiguous
    input segment on an mbarrier) beside the flat one; every candidate
    bit-exact, and the bulk kernel's status word clear."""
    lib = L._lib.load()
    prev = lib.librett_c_set_candidate_set(1)
    rng = np.random.default_rng(11)
    probs = [([4, 6, 128, 5, 16], [3, 0, 4, 2, 1], 16), ([300, 7, 11], [1, 2, 0], 8),
             ([64, 96, 40], [2, 0, 1], 8), ([1024, 512], [1, 0], 4), ([96, 33, 64], [2, 1, 0], 4),
             ([2, 3, 4, 5, 512, 16], [5, 3, 1, 4, 0, 2], 4), ([48, 40, 3, 20], [3, 2, 0, 1], 16),
             ([256, 10, 6, 70], [1, 3, 2, 0], 8)]
    pipes = set()
    try:
        for dims, perm, es in probs:
            n = L.describe(dims, perm, es)["num_candidates"]
            for c in range(n):
                info = _check(dims, perm, es, rng=rng, candidate=c)
                pipes.add(info["pipeline"])
                assert info["status"] == 0, (dims, perm, es, c)
            # 16-byte units fall back to element units for unaligned pointers
            for c in range(n):
                if L.describe(dims, perm, es, candidate=c)["pipeline"] == 3 and es < 16:
                    _check(dims, perm, es, rng=rng, candidate=c, offset=es)
                    break
    finally:
        lib.librett_c_set_candidate_set(prev)
    assert pipes == {0, 1, 2, 3}, pipes


@pytest.mark.parametrize("es", [4, 8, 16])
def test_misaligned_pointers(cuda, es):
    # offsets that keep element alignment but break 16-byte alignment
    rng = np.random.default_rng(es)
    for dims, perm in [([256, 33], [1, 0]), ([100, 3, 40], [0, 2, 1]), ([1 << 12], [0]),
                       ([8, 6, 50], [2, 1, 0])]:
        off = es if es < 16 else 0
        _check(dims, perm, es, rng=rng, offset=off)


def test_plan_measure(cuda):
    rng = np.random.default_rng(3)
    for dims, perm, es in [([64, 48, 32], [2, 0, 1], 4), ([4, 6, 64, 5, 32], [3, 0, 4, 2, 1], 16),
                           ([500, 3, 7], [0, 2, 1], 8)]:
        _check(dims, perm, es, rng=rng, measure=True)


def test_many_streams(cuda):
    """LibreTT test4 analogue: plans on ten streams executing concurrently."""
    import torch

    rng = np.random.default_rng(11)
    streams = [torch.cuda.Stream() for _ in range(10)]
    jobs = []
    for i, s in enumerate(streams):
        dims, perm, es = S.random_problem(rng, max_rank=6, max_vol=1 << 16)
        vol = int(np.prod(dims))
        host = rng.integers(0, 256, vol * es, dtype=np.uint8)
        inp = torch.from_numpy(host).cuda()
        out = torch.zeros_like(inp)
        plan = L.Plan(dims, perm, es, s)
        jobs.append((dims, perm, es, host, inp, out, plan))
    torch.cuda.synchronize()
    for dims, perm, es, host, inp, out, plan in jobs:
        plan.execute(inp.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    for dims, perm, es, host, inp, out, plan in jobs:
        want = O.transpose_np(host, dims, perm, es).view(np.uint8)
        assert np.array_equal(out.cpu().numpy(), want), (dims, perm, es)
        plan.destroy()


def test_error_codes(cuda):
    import torch

    buf = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    out = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    rc, h = L.librettPlan([16, 16], [1, 0], 4, torch.cuda.current_stream())
    assert rc == L.LIBRETT_SUCCESS
    assert L.librettExecute(h, buf.data_ptr(), buf.data_ptr()) == L.LIBRETT_INVALID_PARAMETER
    assert L.librettExecute(h, buf.data_ptr() + 2, out.data_ptr()) == L.LIBRETT_INVALID_PARAMETER
    assert L.librettExecute(h, 0, out.data_ptr()) == L.LIBRETT_INVALID_PARAMETER
    assert L.librettExecute(h, buf.data_ptr(), out.data_ptr()) == L.LIBRETT_SUCCESS
    assert L.librettDestroy(h) == L.LIBRETT_SUCCESS
    assert L.librettDestroy(h) == L.LIBRETT_INVALID_PLAN
    assert L.librettExecute(h, buf.data_ptr(), out.data_ptr()) == L.LIBRETT_INVALID_PLAN
    rc2, h2 = L.librettPlan([16, 16], [1, 0], 4, None)
    assert rc2 == L.LIBRETT_SUCCESS and h2 > h  # handles increase, never reused
    assert L.librettDestroy(h2) == L.LIBRETT_SUCCESS
    for dims, perm, es in [([16, 16], [1, 1], 4), ([16, 0], [1, 0], 4), ([16, 16], [1, 0], 12),
                           ([16], [1], 4)]:
        rc, _ = L.librettPlan(dims, perm, es, None)
        assert rc == L.LIBRETT_INVALID_PARAMETER
    torch.cuda.synchronize()


def _inverse(perm):
    inv = [0] * len(perm)
    for k, p in enumerate(perm):
        inv[p] = k
    return inv


def _sampled_gather_check(inp_words, out_words, dims, perm, nsample, seed):
    """out[o] == in[src(o)] at random output positions, src from LibreTT's
    TensorTester constants (src/TensorTester.cpp:201-220), computed on the GPU."""
    import torch

    rank = len(dims)
    vol = int(np.prod(dims))
    sin = np.cumprod([1] + dims[:-1]).astype(np.int64)
    c = np.zeros(rank, dtype=np.int64)
    c[perm[0]] = 1
    for i in range(1, rank):
        c[perm[i]] = c[perm[i - 1]] * dims[perm[i - 1]]
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    pos = torch.randint(0, vol, (nsample,), device="cuda", generator=g, dtype=torch.int64)
    src = torch.zeros_like(pos)
    for r in range(rank):
        src += ((pos // int(c[r])) % int(dims[r])) * int(sin[r])
    assert torch.equal(out_words[pos], inp_words[src])


@pytest.mark.parametrize("which", ["c3a", "c3b"])
def test_full_size_small_leading_dims(cuda, which):
    """Full-size stress shapes: round trip through the inverse permutation
    returns the input bit-exactly, and sampled outputs obey the gather formula."""
    import torch

    dims, perm, es = S.C3A if which == "c3a" else S.C3B
    vol = int(np.prod(dims))
    words = vol * es // 8
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    inp = torch.randint(-(2 ** 62), 2 ** 62, (words,), device="cuda", dtype=torch.int64,
                        generator=g)
    out = torch.empty_like(inp)
    back = torch.empty_like(inp)
    s = torch.cuda.current_stream()
    odims = [dims[p] for p in perm]
    with L.Plan(dims, perm, es, s) as p1, L.Plan(odims, _inverse(perm), es, s) as p2:
        p1.execute(inp.data_ptr(), out.data_ptr())
        p2.execute(out.data_ptr(), back.data_ptr())
        torch.cuda.synchronize()
    assert torch.equal(back, inp)
    per = es // 8 if es >= 8 else 0
    if es >= 8:
        iw = inp.view(vol, per)
        ow = out.view(vol, per)
    else:
        iw = inp.view(torch.int32)
        ow = out.view(torch.int32)
    _sampled_gather_check(iw, ow, dims, perm, 1 << 20, seed=9)
    del inp, out, back
    torch.cuda.empty_cache()


def test_golden_fixtures(cuda):
    """Engine outputs hash-match the golden fixtures (tests/golden/golden.json)."""
    import hashlib
    import json
    from pathlib import Path

    from tests.golden.make_golden import make_input

    rows = json.loads((Path(__file__).resolve().parent / "golden" / "golden.json").read_text())
    for row in rows:
        dims, perm, es = row["dims"], row["perm"], row["es"]
        inp = make_input(int(np.prod(dims)), es, row["input"])
        got, _ = _run(dims, perm, es, inp)
        assert hashlib.sha256(got.tobytes()).hexdigest() == row["sha256"], row
