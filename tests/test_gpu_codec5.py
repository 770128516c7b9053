"""Codec 5's use of the sorter (src/codecs/bwt_stream.c:46-79, 103-196): the forward with r = bwt_mod + 1 (many
samples on small blocks: r = 8 at 100 bytes), and the decode of blocks below 64 KiB with the primary index only
(kolmo_sais_unbwt, r == n), against the oracle."""
import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec
from kolmo_gb300 import workloads as W
from kolmo_gb300.host import codec5_r

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [100, 4097, 65535, 65536, 300_000, 1 << 21])
def test_codec5_forward_and_inverse(n):
    T = W.markov2(n, 500 + n % 97) if n % 2 else W.zipf_prose(n, 7)
    r = codec5_r(n)
    rc, U, I = codec.bwt_aux(T, r)
    orc, oU, oI = O.bwt_aux(T, r)
    assert rc == 0 and orc == 0
    assert np.array_equal(U, oU) and np.array_equal(I, oI)
    if n < 65536:  # codec 5 stores no samples below 64 KiB: primary index only
        rc, back = codec.unbwt(U, int(I[0]))
    else:
        rc, back = codec.unbwt_aux(U, r, I)
    assert rc == 0 and np.array_equal(back, T)
