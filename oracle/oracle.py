"""CPU oracle for the transpose path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use
this module, always as the checker or as the timed host loop; the engine
never imports it.  Two independent restatements of LibreTT's semantics:

* ``transpose_np``: numpy view/transpose of the column-major tensor, following
  the gather formula of LibreTT tests/example.cpp:170-212;
* ``transpose_c``: the plain-C multithreaded gather loop in oracle/gather.c
  (the CPU baseline), built by ``build_oracle``.

plus the two known-answer checks LibreTT's own tests use:

* ``example_check`` -- the host check of tests/example.cpp:177-212 (for each
  input index compute ``tindex`` and require ``out[tindex] == in[index]``);
* ``pattern_check`` -- the device checker of src/TensorTester.cpp:47-126 with
  the constants of calcTensorConv (src/TensorTester.cpp:201-220), applied to
  outputs of inputs filled with word[w] = w (src/TensorTester.cpp:34-40).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

_WORD = {4: np.uint32, 8: np.uint64, 16: np.dtype([("lo", np.uint64), ("hi", np.uint64)])}


def build_oracle(force: bool = False) -> Path:
    """Compile oracle/gather.c into oracle/_build/liboracle.so with gcc."""
    src = HERE / "gather.c"
    BUILD.mkdir(parents=True, exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread",
                        str(src), "-o", str(tmp)], check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        build_oracle()
        lib = ctypes.CDLL(str(LIB))
        lib.oracle_transpose.restype = ctypes.c_int
        lib.oracle_transpose.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.c_int, ctypes.c_int]
        lib.oracle_check_pattern.restype = ctypes.c_int64
        lib.oracle_check_pattern.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int64),
                                             ctypes.POINTER(ctypes.c_int64)]
        lib.oracle_fill_pattern.restype = None
        lib.oracle_fill_pattern.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        _lib = lib
    return _lib


def _ints(seq):
    arr = (ctypes.c_int * len(seq))(*[int(x) for x in seq])
    return arr


def as_words(buf: np.ndarray, esize: int) -> np.ndarray:
    """View a byte buffer (or any contiguous array) as esize-byte words."""
    return np.ascontiguousarray(buf).view(np.uint8).view(_WORD[esize])


def out_dims(dims, perm):
    return [int(dims[p]) for p in perm]


def transpose_np(buf: np.ndarray, dims, perm, esize: int) -> np.ndarray:
    """numpy restatement; returns the output as a flat array of esize-byte words."""
    rank = len(dims)
    w = as_words(buf, esize)
    vol = int(np.prod(dims, dtype=np.int64))
    assert w.size == vol, (w.size, vol)
    a = w.reshape(tuple(int(d) for d in dims[::-1]))  # column-major view
    axes = [rank - 1 - perm[rank - 1 - k] for k in range(rank)]
    return np.ascontiguousarray(a.transpose(axes)).reshape(-1)


def transpose_c(buf: np.ndarray, dims, perm, esize: int, nthreads: int = 1,
                out: np.ndarray | None = None) -> np.ndarray:
    """Plain-C gather loop (oracle/gather.c); returns esize-byte words."""
    lib = _load()
    src = np.ascontiguousarray(buf).view(np.uint8)
    if out is None:
        out = np.empty(src.nbytes, dtype=np.uint8)
    dst = out.view(np.uint8)
    assert dst.nbytes == src.nbytes
    rc = lib.oracle_transpose(src.ctypes.data, dst.ctypes.data, len(dims), _ints(dims),
                              _ints(perm), esize, nthreads)
    if rc != 0:
        raise ValueError("oracle_transpose rejected its arguments")
    return dst.view(_WORD[esize])


def fill_pattern(nbytes: int) -> np.ndarray:
    """uint8 buffer whose 32-bit words hold their own index."""
    assert nbytes % 4 == 0
    return np.arange(nbytes // 4, dtype=np.uint32).view(np.uint8)


def pattern_check(out: np.ndarray, dims, perm, esize: int):
    """LibreTT's TensorTester check; returns (first_bad_pos, ref, data) or None."""
    lib = _load()
    o = np.ascontiguousarray(out).view(np.uint8)
    ref = ctypes.c_int64(0)
    dat = ctypes.c_int64(0)
    pos = lib.oracle_check_pattern(o.ctypes.data, len(dims), _ints(dims), _ints(perm), esize,
                                   ctypes.byref(ref), ctypes.byref(dat))
    if pos == -2:
        raise ValueError("oracle_check_pattern rejected its arguments")
    return None if pos == -1 else (int(pos), int(ref.value), int(dat.value))


def example_check(inp: np.ndarray, out: np.ndarray, dims, perm, esize: int) -> bool:
    """LibreTT tests/example.cpp:177-212 host check, vectorised with numpy."""
    rank = len(dims)
    vin = as_words(inp, esize)
    vout = as_words(out, esize)
    vol = vin.size
    abc = np.ones(rank, dtype=np.int64)
    cba = np.ones(rank, dtype=np.int64)
    for i in range(1, rank):
        abc[i] = abc[i - 1] * dims[i - 1]
        cba[i] = cba[i - 1] * dims[perm[i - 1]]
    index = np.arange(vol, dtype=np.int64)
    rem = index.copy()
    ijk = np.zeros((rank, vol), dtype=np.int64)
    for r in range(rank - 1, -1, -1):
        ijk[r] = rem // abc[r]
        rem -= abc[r] * ijk[r]
    tindex = np.zeros(vol, dtype=np.int64)
    for r in range(rank):
        tindex += cba[r] * ijk[perm[r]]
    return bool(np.array_equal(vout[tindex], vin[index]))
