"""Seeded problem generators for batched (grouped) execution.

A problem is (dims, perm, element_bytes) in LibreTT's column-major
convention.  The batch distribution: rank uniform in 2..6; volume
log-uniform in [2^lo, 2^hi] elements; dims split the volume with random
log-weights (each >= 2, product within 5% of the drawn volume); element size
4 or 8 bytes with equal probability; a uniformly random permutation.
"""
from __future__ import annotations

import numpy as np

GROUPED_SEED = 20270304


def grouped_problems(n=10000, seed=GROUPED_SEED, log2_lo=10.0, log2_hi=22.0, sizes=(4, 8),
                     max_rank=6):
    rng = np.random.Generator(np.random.MT19937(seed))
    out = []
    for _ in range(n):
        rank = int(rng.integers(2, max_rank + 1))
        lv = float(rng.uniform(log2_lo, log2_hi))
        target = 2.0 ** lv
        w = rng.uniform(0.0, 1.0, rank)
        logd = w / w.sum() * lv
        dims = [max(2, int(round(2.0 ** x))) for x in logd]
        for _ in range(64):
            vol = float(np.prod(dims, dtype=np.float64))
            if abs(vol - target) <= 0.05 * target:
                break
            i = int(np.argmax(dims))
            nd = max(2, int(round(dims[i] * target / vol)))
            if nd == dims[i]:
                break
            dims[i] = nd
        perm = [int(x) for x in rng.permutation(rank)]
        es = int(sizes[int(rng.integers(0, len(sizes)))])
        out.append((dims, perm, es))
    return out


def packed_offsets(problems, align=256):
    """Byte offset of each problem's tensor in one buffer (each start aligned
    to `align` bytes) and the buffer's total size."""
    offs, total = [], 0
    for dims, _, es in problems:
        offs.append(total)
        nb = int(np.prod(dims)) * es
        total += (nb + align - 1) // align * align
    return offs, max(total, align)
