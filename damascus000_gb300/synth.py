"""Seeded synthetic workloads for the Damascus Fold benchmarks.

Inputs are uniformly random bytes from a ChaCha20 keystream (RFC 8439 block
function, written here with numpy and vectorised over blocks) keyed by a
master seed, so every run of a workload sees the same files and seeds.  No
public dataset is involved: the reference benchmarks synthetic files only.

Per file, bytes [0, L) are the file and the next 32 bytes are
SystemParams.seed_generators (src/utils/config.rs:24-44).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np

_SIGMA = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)


def _rotl(x: np.ndarray, n: int) -> np.ndarray:
    return (x << np.uint32(n)) | (x >> np.uint32(32 - n))


def chacha20_stream(key: bytes, nbytes: int, nonce: bytes = bytes(12), counter: int = 0) -> bytes:
    """ChaCha20 keystream (20 rounds, 32-bit counter, 96-bit nonce)."""
    assert len(key) == 32 and len(nonce) == 12
    nblocks = (nbytes + 63) // 64
    if nblocks == 0:
        return b""
    k = np.frombuffer(key, dtype="<u4").astype(np.uint32)
    nn = np.frombuffer(nonce, dtype="<u4").astype(np.uint32)
    st = np.empty((16, nblocks), dtype=np.uint32)
    st[0:4] = _SIGMA[:, None]
    st[4:12] = k[:, None]
    st[12] = (np.arange(nblocks, dtype=np.uint64) + counter).astype(np.uint32)
    st[13:16] = nn[:, None]
    x = st.copy()

    def qr(a, b, c, d):
        x[a] += x[b]; x[d] ^= x[a]; x[d] = _rotl(x[d], 16)
        x[c] += x[d]; x[b] ^= x[c]; x[b] = _rotl(x[b], 12)
        x[a] += x[b]; x[d] ^= x[a]; x[d] = _rotl(x[d], 8)
        x[c] += x[d]; x[b] ^= x[c]; x[b] = _rotl(x[b], 7)

    with np.errstate(over="ignore"):
        for _ in range(10):
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
        x += st
    return x.T.astype("<u4").tobytes()[:nbytes]


def _derive_key(master_seed: int, label: str, index: int) -> bytes:
    base = master_seed.to_bytes(8, "little") + index.to_bytes(8, "little")
    lab = label.encode()[:16].ljust(16, b"\0")
    return base + lab


def random_file(master_seed: int, length: int, index: int = 0):
    """(file bytes, seed_generators) for file ``index`` of a workload."""
    s = chacha20_stream(_derive_key(master_seed, "file", index), length + 32)
    return s[:length], s[length:length + 32]


class _Uniform:
    """Deterministic uniform doubles in [0, 1) from a ChaCha20 stream."""

    def __init__(self, master_seed: int, label: str, count: int):
        raw = np.frombuffer(chacha20_stream(_derive_key(master_seed, label, 0), 8 * max(count, 1)), dtype="<u8")
        self.v = (raw >> np.uint64(11)).astype(np.float64) / float(1 << 53)
        self.i = 0

    def next(self) -> float:
        u = float(self.v[self.i])
        self.i += 1
        return u


def log_uniform_sizes(master_seed: int, count: int, lo: int, hi: int, label: str = "sizes") -> List[int]:
    u = _Uniform(master_seed, label, count)
    return [int(round(math.exp(math.log(lo) + u.next() * (math.log(hi) - math.log(lo))))) for _ in range(count)]


@dataclass
class Request:
    index: int
    arrival_s: float
    size: int


def serving_stream(master_seed: int, count: int, rate_per_s: float = 200.0) -> List[Request]:
    """Poisson arrivals; sizes 50% log-uniform 50 KB-1 MiB, 40% 1-8 MiB, 10% 16 MiB."""
    u = _Uniform(master_seed, "serve", 3 * count)
    t = 0.0
    out = []
    for i in range(count):
        t += -math.log(1.0 - u.next()) / rate_per_s
        b = u.next()
        r = u.next()
        if b < 0.5:
            lo, hi = 50_000, 1 << 20
        elif b < 0.9:
            lo, hi = 1 << 20, 8 << 20
        else:
            lo, hi = 16 << 20, 16 << 20
        size = int(round(math.exp(math.log(lo) + r * (math.log(hi) - math.log(lo)))))
        out.append(Request(i, t, size))
    return out


def serving_files(master_seed: int, count: int, rate_per_s: float = 200.0, seed_generators: bytes = None):
    """[(file bytes, seed_generators, arrival_s)] of the serving stream.

    File ``i`` is ``random_file(master_seed, size_i, 10_000 + i)``; with
    ``seed_generators`` given, every file uses that one system seed instead of
    its own (SystemParams::default, src/utils/config.rs:19, 33-44)."""
    out = []
    for r in serving_stream(master_seed, count, rate_per_s):
        data, seed = random_file(master_seed, r.size, 10_000 + r.index)
        out.append((data, seed_generators if seed_generators is not None else seed, r.arrival_s))
    return out


def batched_files(master_seed: int, count: int, lo: int, hi: int):
    """[(file bytes, seed_generators, 0.0)] of the batched set: log-uniform sizes in
    [lo, hi], file ``i`` = ``random_file(master_seed, size_i, 20_000 + i)``."""
    sizes = log_uniform_sizes(master_seed, count, lo, hi)
    return [random_file(master_seed, n, 20_000 + i) + (0.0,) for i, n in enumerate(sizes)]
