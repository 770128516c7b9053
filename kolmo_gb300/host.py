"""Host-side rules of the reference's callers of the BWT path, restated so that the GPU path is driven with exactly
the sampling intervals the codecs use (adnaneben/kolmo src/codecs/bwt_stream.c).

* ``bwt_mod``: libbsc's sampling interval minus one, the largest power of two <= n / 8, minus one
  (bwt_stream.c:40-45).
* ``codec18_rlog``: codec 18's log2 of the sampling interval (bwt_stream.c:224-227): bwt_mod's power (at least 1),
  raised until at most 255 sampled indexes follow the primary index.
* ``codec5_r``: codec 5's interval, bwt_mod + 1 (bwt_stream.c:50-52).
"""
from __future__ import annotations


def bwt_mod(n: int) -> int:
    mod = n // 8
    mod |= mod >> 1
    mod |= mod >> 2
    mod |= mod >> 4
    mod |= mod >> 8
    mod |= mod >> 16
    return mod >> 1


def codec18_rlog(lz: int, index_log2: int = 0) -> int:
    rlog = index_log2 if index_log2 > 0 else 0
    if not rlog:
        mod = bwt_mod(lz)
        rlog = 0
        while (2 << rlog) <= mod + 1:
            rlog += 1
        if rlog < 1:
            rlog = 1
    elif rlog < 1:
        rlog = 1
    while rlog < 30 and ((lz - 1) >> rlog) > 255:
        rlog += 1
    return rlog


def codec5_r(n: int) -> int:
    return bwt_mod(n) + 1


def n_samples(n: int, r: int) -> int:
    """Entries of I for a block of n bytes: the primary index plus k = (n - 1) / r samples."""
    return (n - 1) // r + 1 if n > 0 else 1
