"""Problem shapes shared by the tests.

TEST3 lists the hand-picked shapes of LibreTT tests/librett_test.cpp:277-417
(each run there for 4- and 8-byte elements); EXAMPLE is the shape of
tests/example.cpp:88-89 (run for 4, 8 and 16 bytes).
"""
import itertools

import numpy as np

EXAMPLE = ([3, 3, 3, 2, 4], [1, 3, 0, 4, 2])

TEST3 = [
    ([43, 67], [1, 0]),
    ([65536 * 32, 2], [1, 0]),
    ([1305, 599, 88], [0, 2, 1]),
    ([24, 330, 64, 147], [1, 0, 2, 3]),
    ([2, 5, 9, 12], [0, 1, 2, 3]),
    ([2, 4, 6, 9, 11, 13], [0, 1, 2, 3, 4, 5]),
    ([5, 42, 75, 86, 57], [1, 3, 4, 2, 0]),
    ([5, 3, 2, 9, 14], [0, 1, 3, 2, 4]),
]

# Small-leading-dimension stress shapes (full size).
C3A = ([4, 6, 8192, 5, 256], [3, 0, 4, 2, 1], 16)
C3B = ([2, 3, 4, 5, 65536, 16], [5, 3, 1, 4, 0, 2], 4)
C1 = ([64, 48, 32], [2, 0, 1], 4)


def test1_dims(rank):
    """Dims of LibreTT test1 (tests/librett_test.cpp:168-188): 2 + r*14/rank."""
    return [2 + r * 14 // rank for r in range(rank)]


def test1_cases(max_rank=7, max_perms_per_rank=None, seed=0):
    rng = np.random.default_rng(seed)
    for rank in range(2, max_rank + 1):
        perms = list(itertools.permutations(range(rank)))
        if max_perms_per_rank is not None and len(perms) > max_perms_per_rank:
            idx = rng.choice(len(perms), size=max_perms_per_rank, replace=False)
            perms = [perms[i] for i in sorted(idx)]
        for p in perms:
            yield test1_dims(rank), list(p)


def random_problem(rng, max_rank=8, max_vol=1 << 20, min_dim=1):
    """Seeded random shape in the spirit of LibreTT test2 (tests/librett_test.cpp:194-272)."""
    rank = int(rng.integers(2, max_rank + 1))
    logvol = rng.uniform(np.log(max(8, 2 ** rank)), np.log(max_vol))
    w = rng.uniform(0.05, 1.0, rank)
    logd = w / w.sum() * logvol
    dims = [max(min_dim, int(round(np.exp(x)))) for x in logd]
    while int(np.prod(dims)) > max_vol:
        i = int(np.argmax(dims))
        dims[i] = max(1, dims[i] // 2)
    perm = [int(x) for x in rng.permutation(rank)]
    es = int(rng.choice([4, 8, 16]))
    return dims, perm, es
