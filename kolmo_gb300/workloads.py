"""Seeded synthetic inputs for the BWT path (bindings to ``csrc/workloads.c``).

Sources: order-2 Markov bytes over 64 symbols with Dirichlet(0.3) rows, Zipf(1.1) word prose with verbatim repeats, ACGT with 0.1% N, templated log lines, periodic
text with one flip per MiB and the Fibonacci word; plus the size distributions of the mixed batch (log-uniform
16 KiB-16 MiB) and of the request stream (lognormal, median 256 KiB, sigma 1.5, capped at 128 MiB). The same seed
gives the same bytes on every machine.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_P = ctypes.c_void_p
_U64 = ctypes.c_uint64


def lib():
    global _lib
    if _lib is None:
        path = _build.WORKLOADS
        if not os.path.exists(path):
            _build.build_workloads()
        L = ctypes.CDLL(path)
        L.kgw_markov2.argtypes = [_P, _U64, _U64, ctypes.c_int, ctypes.c_double]
        L.kgw_zipf_prose.argtypes = [_P, _U64, _U64, ctypes.c_int, ctypes.c_double, ctypes.c_uint32, ctypes.c_int,
                                     ctypes.c_uint32, ctypes.c_uint32]
        L.kgw_acgt.argtypes = [_P, _U64, _U64, ctypes.c_uint32]
        L.kgw_logs.argtypes = [_P, _U64, _U64]
        L.kgw_periodic.argtypes = [_P, _U64, _U64, _U64, _U64]
        L.kgw_fibonacci.argtypes = [_P, _U64]
        L.kgw_loguniform_sizes.argtypes = [_U64, ctypes.c_int, _U64, _U64, _P]
        L.kgw_requests.argtypes = [_U64, ctypes.c_int, ctypes.c_double, ctypes.c_double, _U64, ctypes.c_double,
                                   _P, _P, _P, _P]
        L.kgw_source_block.argtypes = [ctypes.c_int, _P, _U64, _U64]
        L.kgw_fnv1a.argtypes = [_P, _U64]
        L.kgw_fnv1a.restype = _U64
        for f in ("kgw_markov2", "kgw_zipf_prose", "kgw_acgt", "kgw_logs", "kgw_periodic", "kgw_fibonacci",
                  "kgw_source_block"):
            getattr(L, f).restype = ctypes.c_int
        _lib = L
    return _lib


def _buf(n: int, out: np.ndarray | None):
    if out is None:
        out = np.empty(max(n, 1), np.uint8)
    return out


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc})")


def markov2(n: int, seed: int, nsym: int = 64, alpha: float = 0.3, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_markov2(out.ctypes.data, n, seed, nsym, alpha), "markov2")
    return out[:n]


def zipf_prose(n: int, seed: int, vocab: int = 50000, s: float = 1.1, noise_ppm: int = 20000, ncopies: int = 200,
               copy_min: int = 4096, copy_max: int = 65536, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_zipf_prose(out.ctypes.data, n, seed, vocab, s, noise_ppm, ncopies, copy_min, copy_max),
           "zipf_prose")
    return out[:n]


def acgt(n: int, seed: int, n_ppm: int = 1000, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_acgt(out.ctypes.data, n, seed, n_ppm), "acgt")
    return out[:n]


def logs(n: int, seed: int, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_logs(out.ctypes.data, n, seed), "logs")
    return out[:n]


def periodic(n: int, seed: int, period: int, flip_every: int = 1 << 20, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_periodic(out.ctypes.data, n, seed, period, flip_every), "periodic")
    return out[:n]


def fibonacci(n: int, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_fibonacci(out.ctypes.data, n), "fibonacci")
    return out[:n]


SOURCES = ("markov", "acgt", "logs")


def source_block(source: int, n: int, seed: int, out=None) -> np.ndarray:
    out = _buf(n, out)
    _check(lib().kgw_source_block(source, out.ctypes.data, n, seed), "source_block")
    return out[:n]


def loguniform_sizes(seed: int, count: int, lo: int, hi: int) -> np.ndarray:
    s = np.zeros(count, np.uint64)
    lib().kgw_loguniform_sizes(seed, count, lo, hi, s.ctypes.data)
    return s


def requests(seed: int, count: int, median: float = 256 * 1024, sigma: float = 1.5, cap: int = 128 << 20,
             rate: float = 100.0):
    """Request stream: (sizes, inter-arrival gaps in s, mix draws in [0,1000), source ids in [0,3))."""
    sizes = np.zeros(count, np.uint64)
    gaps = np.zeros(count, np.float64)
    mix = np.zeros(count, np.uint32)
    src = np.zeros(count, np.uint32)
    lib().kgw_requests(seed, count, median, sigma, cap, rate, sizes.ctypes.data, gaps.ctypes.data, mix.ctypes.data,
                       src.ctypes.data)
    return sizes, gaps, mix, src


def fnv1a(a: np.ndarray) -> int:
    b = np.ascontiguousarray(a).view(np.uint8).ravel()
    return int(lib().kgw_fnv1a(b.ctypes.data, b.size))


# ---- the benchmark workloads (seeded; sizes as the benchmark configurations state them)
SEED_MARKOV_1MIB = 0x4B4F4C4D4F0001
SEED_PROSE_64MIB = 0x4B4F4C4D4F0002
SEED_BATCH = 0x4B4F4C4D4F0003
SEED_DEGENERATE = 0x4B4F4C4D4F0004
SEED_SERVE = 0x4B4F4C4D4F0005


def markov_1mib() -> np.ndarray:
    """1 MiB order-2 Markov block over a 64-symbol byte alphabet, Dirichlet(0.3) rows."""
    return markov2(1 << 20, SEED_MARKOV_1MIB)


def prose_64mib(n: int = 64 << 20) -> np.ndarray:
    """64 MiB Zipf(1.1) word prose, 50k-word vocabulary, 2% random bytes, 200 verbatim 4-64 KiB repeats."""
    return zipf_prose(n, SEED_PROSE_64MIB)


def mixed_batch(count: int = 256, lo: int = 16 << 10, hi: int = 16 << 20, seed: int = SEED_BATCH):
    """The mixed batch: count blocks, log-uniform sizes, each from one of the three sources (round robin on a seeded
    draw). Returns a list of (source, array)."""
    sizes = loguniform_sizes(seed, count, lo, hi)
    out = []
    for i, n in enumerate(sizes):
        src = int((seed >> 3) + i * 0x9E37) % 3
        out.append((src, source_block(src, int(n), seed * 1000003 + i)))
    return out


def degenerate(kind: str, n: int = 128 << 20) -> np.ndarray:
    """periodic-1, periodic-7, periodic-4096 (one random flip per MiB) or fibonacci."""
    if kind == "fibonacci":
        return fibonacci(n)
    period = int(kind.split("-")[1])
    return periodic(n, SEED_DEGENERATE + period, period, 1 << 20)
