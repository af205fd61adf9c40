"""Generate the golden transpose fixtures in tests/golden/.

Run from the repository root:  python tests/golden/make_golden.py

The expected outputs are computed with the host check of LibreTT
tests/example.cpp:177-212, restated here on its own (numpy, vectorised):
for every input index, decompose it with abc[] into ijk[], form
tindex = sum_r cba[r] * ijk[perm[r]], and place in[index] at out[tindex].

Inputs follow LibreTT's two test conventions:
  "value": element i holds i in the element type (int32 / int64 /
           complex<double>(i, 0)), as tests/example.cpp:150-152 does;
  "words": 32-bit word w holds w, as src/TensorTester.cpp:34-40 does.

Outputs: golden.json (sha256 of every expected output) and example_<es>.npy
(full expected outputs of the example shape).
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from tests import shapes as S  # noqa: E402


def make_input(vol, es, kind):
    if kind == "words":
        return np.arange(vol * es // 4, dtype=np.uint32).view(np.uint8)
    i = np.arange(vol, dtype=np.int64)
    if es == 4:
        return i.astype(np.int32).view(np.uint8)
    if es == 8:
        return i.view(np.uint8)
    c = np.zeros(vol, dtype=np.complex128)
    c.real = i
    return c.view(np.uint8)


def expected(inp, dims, perm, es):
    rank = len(dims)
    vol = int(np.prod(dims))
    words = inp.reshape(vol, es)
    abc = [1] * rank
    cba = [1] * rank
    for i in range(1, rank):
        abc[i] = abc[i - 1] * dims[i - 1]
        cba[i] = cba[i - 1] * dims[perm[i - 1]]
    index = np.arange(vol, dtype=np.int64)
    rem = index.copy()
    ijk = [None] * rank
    for r in range(rank - 1, -1, -1):
        ijk[r] = rem // abc[r]
        rem = rem - abc[r] * ijk[r]
    tindex = np.zeros(vol, dtype=np.int64)
    for r in range(rank):
        tindex += cba[r] * ijk[perm[r]]
    out = np.empty_like(words)
    out[tindex] = words[index]
    return out.reshape(-1)


def cases():
    dims, perm = S.EXAMPLE
    for es in (4, 8, 16):
        for kind in ("value", "words"):
            yield dims, perm, es, kind
    for dims, perm in S.TEST3:
        for es in (4, 8):
            yield dims, perm, es, "value"
    yield S.C1[0], S.C1[1], 4, "value"
    for dims, perm in S.test1_cases(max_rank=4):
        yield dims, perm, 8, "words"


def main():
    rows = []
    for dims, perm, es, kind in cases():
        vol = int(np.prod(dims))
        inp = make_input(vol, es, kind)
        out = expected(inp, dims, perm, es)
        rows.append({"dims": dims, "perm": perm, "es": es, "input": kind,
                     "nbytes": int(out.nbytes), "sha256": hashlib.sha256(out.tobytes()).hexdigest()})
    (HERE / "golden.json").write_text(json.dumps(rows, indent=1) + "\n")
    dims, perm = S.EXAMPLE
    for es in (4, 8, 16):
        vol = int(np.prod(dims))
        np.save(HERE / f"example_{es}.npy", expected(make_input(vol, es, "value"), dims, perm, es))
    print(f"wrote {len(rows)} golden rows")


if __name__ == "__main__":
    main()
