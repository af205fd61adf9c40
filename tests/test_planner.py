"""Host planner invariants (CPU only, through librett_c_describe)."""
import itertools

import numpy as np
import pytest

import librett_gb300 as L
from tests import shapes as S


def _mapping(dims, perm):
    """out position of every input element, by LibreTT's gather formula."""
    rank = len(dims)
    vol = int(np.prod(dims))
    a = np.arange(vol, dtype=np.int64).reshape(tuple(dims[::-1]))
    axes = [rank - 1 - perm[rank - 1 - k] for k in range(rank)]
    src_of_out = np.ascontiguousarray(a.transpose(axes)).reshape(-1)
    out_of_src = np.empty(vol, dtype=np.int64)
    out_of_src[src_of_out] = np.arange(vol)
    return out_of_src


def _check_plan(dims, perm, es, candidate=-1):
    info = L.describe(dims, perm, es, candidate=candidate)
    fd, fp, ext = info["fused_dim"], info["fused_perm"], info["tile_extent"]
    vol = int(np.prod(dims))
    assert info["volume"] == vol == int(np.prod(fd))
    assert sorted(fp) == list(range(len(fd)))
    # the fused problem is the same permutation of linear indices
    if vol <= 1 << 22:
        assert np.array_equal(_mapping(fd, fp), _mapping(dims, perm))
    # no two neighbouring fused ranks could have been fused further
    for i in range(1, len(fp)):
        assert fp[i] != fp[i - 1] + 1
    assert all(d > 1 for d in fd) or fd == [1]
    m = info["method"]
    if m == 1:  # Trivial
        assert len(fd) == 1
        return info
    if m == 5:  # TiledCopy
        assert fp[0] == 0
        return info
    # tile kernels: extents, tiles, slots and smem are consistent
    assert all(1 <= e <= d for e, d in zip(ext, fd))
    tvol = int(np.prod(ext))
    lv = info["unit_in_bytes"] // es
    sv = info["unit_out_bytes"] // es
    assert lv in (1, 16 // es) and sv in (1, 16 // es)
    assert tvol % lv == 0 and tvol % sv == 0
    assert tvol <= 4096 and info["slots"] * info["threads"] * lv >= tvol
    assert info["slots"] in (1, 2, 4, 8, 16)
    assert info["num_tiles"] == int(np.prod([-(-d // e) for d, e in zip(fd, ext)]))
    assert info["smem_bytes"] <= 227 * 1024
    buffers = 1 if info["pipeline"] in (2, 3) else 2  # one-tile-per-CTA pipelines: one buffer
    assert info["smem_bytes"] >= buffers * tvol * es
    ragged = sum(1 for d, e in zip(fd, ext) if d % e)
    assert ragged <= 2
    # Every element is covered by a full tile; a ragged rank's last chunk
    # starts at dim - extent, so chunks overlap by less than one chunk count
    # along that rank (small problems only).
    if vol <= 1 << 16:
        sin = np.cumprod([1] + fd[:-1])
        seen = np.zeros(vol, dtype=np.int64)
        chunks = [range(-(-d // e)) for d, e in zip(fd, ext)]
        for c in itertools.product(*chunks):
            lo = [min(ci * e, d - e) for ci, e, d in zip(c, ext, fd)]
            grids = np.meshgrid(*[np.arange(l, l + e) for l, e in zip(lo, ext)], indexing="ij")
            idx = sum(g.astype(np.int64) * s for g, s in zip(grids, sin))
            np.add.at(seen, idx.reshape(-1), 1)
        assert (seen >= 1).all()
        tiles_total = int(np.prod([len(r) for r in chunks])) * tvol
        assert seen.sum() == tiles_total
        overlap = tiles_total / vol - 1.0
        bound = 1.0
        for d, e in zip(fd, ext):
            nch = -(-d // e)
            bound *= nch * e / d
        assert overlap <= bound - 1.0 + 1e-9
    return info


def test_reference_shapes_plan():
    for dims, perm in S.TEST3 + [S.EXAMPLE]:
        for es in (4, 8, 16):
            _check_plan(dims, perm, es)
    for dims, perm, es in (S.C1, S.C3A, S.C3B):
        _check_plan(dims, perm, es)


def test_c1_fuses_to_2d():
    info = L.describe(*S.C1)
    assert info["fused_dim"] == [3072, 32] and info["fused_perm"] == [1, 0]
    assert info["method"] == 4  # Tiled


def test_small_leading_dims_do_not_fuse():
    for dims, perm, es in (S.C3A, S.C3B):
        info = L.describe(dims, perm, es)
        assert info["fused_dim"] == dims and info["fused_perm"] == perm
        assert info["run_in_bytes"] >= 256 and info["run_out_bytes"] >= 256


def test_random_shapes_all_candidates():
    rng = np.random.default_rng(123)
    for _ in range(60):
        dims, perm, es = S.random_problem(rng, max_rank=7, max_vol=1 << 14)
        n = L.describe(dims, perm, es)["num_candidates"]
        for c in range(n):
            _check_plan(dims, perm, es, candidate=c)


def test_unit_dims_dropped():
    info = L.describe([1, 7, 1, 5], [3, 2, 1, 0], 4)
    assert info["fused_dim"] == [7, 5] and info["fused_perm"] == [1, 0]
    assert L.describe([1, 1], [1, 0], 8)["method"] == 1
    assert L.describe([3, 4, 5], [0, 1, 2], 16)["method"] == 1


def _fastdiv(n, d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << (31 + l)) // d) + 1
    assert m < (1 << 32)
    return (n * m) >> (31 + l)


def test_fast_division_formula():
    rng = np.random.default_rng(0)
    ds = list(range(1, 1100)) + [2 ** k for k in range(32)] + [2 ** k - 1 for k in range(2, 32)]
    ds += [2 ** k + 1 for k in range(1, 31)] + [int(x) for x in rng.integers(1, 2 ** 31, 400)]
    for d in ds:
        ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, 2 ** 31 - 1, 2 ** 31 - 2]
        ns += [int(x) for x in rng.integers(0, 2 ** 31, 20)]
        for n in ns:
            if 0 <= n < 2 ** 31:
                assert _fastdiv(n, d) == n // d, (n, d)


def test_umulhi_digit_exact():
    """The flat and bulk-copy kernels take the digits of in-tile indices
    (< 2^16) by __umulhi(x, ceil(2^32 / e)) for extents e >= 2; exhaustive
    over e <= 4096 (the largest tile volume) and x < 2^16."""
    x = np.arange(1 << 16, dtype=np.uint64)
    for e in range(2, 4097):
        m = np.uint64(((1 << 32) + e - 1) // e)
        assert np.array_equal((x * m) >> np.uint64(32), x // np.uint64(e)), e
