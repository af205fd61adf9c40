"""Seeded random-bit test inputs and the output digest -- TEST INFRASTRUCTURE.

The parity fixtures at benchmark sizes (tests/golden/librett_random.json)
hold, per case, the digest of LibreTT's own output for an input defined
here, so the engine's output can be compared with LibreTT's without storing
gigabytes.  The same definitions are restated in C++ in
oracle/ref_bench/ref_driver.cpp (the program that runs LibreTT's build).

Input: the tensor's bytes are the little-endian 64-bit words
    w[i] = mix64(key + (i + 1) * 0x9E3779B97F4A7C15),  i = 0, 1, ...
truncated to vol * sizeofType bytes, where mix64 is the SplitMix64 output
function (Steele, Lea and Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014):
    z ^= z >> 30; z *= 0xBF58476D1CE4E5B9; z ^= z >> 27; z *= 0x94D049BB133111EB;
    z ^= z >> 31
(all arithmetic mod 2^64).  Every bit pattern occurs, NaN and Inf payloads
included, so a transpose that moves values as floating point would show.

Digest: sha256 of the concatenated sha256 digests of consecutive 64 MiB
chunks of the output (the last chunk may be shorter).  Chunks hash in
parallel, which keeps multi-gigabyte outputs cheap to check.
"""
from __future__ import annotations

import hashlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np

GOLDEN = 0x9E3779B97F4A7C15
M1 = 0xBF58476D1CE4E5B9
M2 = 0x94D049BB133111EB
CHUNK = 64 << 20


def _s64(x: int) -> int:
    """A 64-bit pattern as a signed int64 value."""
    return x - (1 << 64) if x >= 1 << 63 else x


def words_np(key: int, start: int, n: int) -> np.ndarray:
    """w[start .. start + n) as uint64 (numpy, host)."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(key) + i * np.uint64(GOLDEN)
        z ^= z >> np.uint64(30)
        z *= np.uint64(M1)
        z ^= z >> np.uint64(27)
        z *= np.uint64(M2)
        z ^= z >> np.uint64(31)
    return z


def _lsr(z, k: int):
    """Logical right shift of int64 torch values."""
    return (z >> k) & ((1 << (64 - k)) - 1)


def fill_torch(buf_u8, key: int, chunk_words: int = 1 << 26) -> None:
    """Writes the input bytes for `key` into a torch uint8 tensor (any
    device), chunk by chunk.  int64 arithmetic wraps mod 2^64 in torch, so
    the words equal words_np's bit for bit."""
    import torch

    nbytes = buf_u8.numel()
    nwords = (nbytes + 7) // 8
    dev = buf_u8.device
    for w0 in range(0, nwords, chunk_words):
        n = min(chunk_words, nwords - w0)
        z = torch.arange(w0 + 1, w0 + n + 1, dtype=torch.int64, device=dev)
        z = z * _s64(GOLDEN) + _s64(key % (1 << 64))
        z = z ^ _lsr(z, 30)
        z = z * _s64(M1)
        z = z ^ _lsr(z, 27)
        z = z * _s64(M2)
        z = z ^ _lsr(z, 31)
        b0 = 8 * w0
        b1 = min(nbytes, b0 + 8 * n)
        buf_u8[b0:b1] = z.view(torch.uint8)[:b1 - b0]


def input_bytes(key: int, nbytes: int) -> np.ndarray:
    """The input bytes for `key` (host)."""
    return words_np(key, 0, (nbytes + 7) // 8).view(np.uint8)[:nbytes].copy()


def tree_digest(data, threads: int = 16) -> str:
    """Digest of a bytes-like object (numpy uint8 array, bytes, memoryview)."""
    mv = memoryview(np.ascontiguousarray(data).view(np.uint8)).cast("B")
    chunks = [mv[o:o + CHUNK] for o in range(0, len(mv), CHUNK)] or [mv[0:0]]
    with ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(lambda c: hashlib.sha256(c).digest(), chunks))
    return hashlib.sha256(b"".join(parts)).hexdigest()


class StreamDigest:
    """tree_digest over data that arrives in pieces (for example through a
    pipe): equal to tree_digest of the concatenation."""

    def __init__(self, threads: int = 16):
        self._ex = ThreadPoolExecutor(max_workers=threads)
        self._futs = []
        self._buf = bytearray()
        self._n = 0

    def update(self, piece) -> None:
        self._buf += piece
        self._n += len(piece)
        while len(self._buf) >= CHUNK:
            c = bytes(self._buf[:CHUNK])
            del self._buf[:CHUNK]
            self._futs.append(self._ex.submit(lambda c=c: hashlib.sha256(c).digest()))

    def hexdigest(self) -> str:
        if self._buf or not self._futs:
            c = bytes(self._buf)
            self._futs.append(self._ex.submit(lambda c=c: hashlib.sha256(c).digest()))
            self._buf = bytearray()
        parts = [f.result() for f in self._futs]
        self._ex.shutdown()
        return hashlib.sha256(b"".join(parts)).hexdigest()
