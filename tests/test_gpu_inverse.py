"""Inverse BWT on the GPU: decodes the reference's BWT strings (checked against the golden hashes first) back to
the exact input; the r == n path (kolmo_sais_unbwt); range checks; strings that are not a valid BWT."""
import numpy as np
import pytest

import oracle as O
from golden_cases import h, make_input
from kolmo_gb300 import codec, native
from kolmo_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_inverse_restores_golden_inputs(golden):
    for c in golden:
        T = make_input(c)
        rc, U, I = O.bwt_aux(T, c["r"])
        assert h(U) == c["U"] and h(I.astype("<i4")) == c["I"]  # the reference's BWT
        rc, back = codec.unbwt_aux(U, c["r"], I)
        assert rc == 0, (c["name"], native.last_error())
        assert np.array_equal(back, T), c["name"]
        rc, back = codec.unbwt(U, int(I[0]))
        assert rc == 0 and np.array_equal(back, T), c["name"]


def test_inverse_batch_uneven_sizes():
    rng = np.random.default_rng(9)
    blocks, texts = [], []
    for i in range(40):
        n = int(2 ** rng.uniform(1, 21))
        T = W.source_block(i % 3, n, 100 + i)
        rc, U, I = O.bwt_aux(T, 1 << 10)
        blocks.append((U, 1 << 10, I))
        texts.append(T)
    rc, res = codec.inv_batch(blocks)
    assert rc == 0, native.last_error()
    for T, (brc, back) in zip(texts, res):
        assert brc == 0 and np.array_equal(back, T)


def test_inverse_out_of_range_index_refused():
    T = W.markov2(5000, 1)
    rc, U, I = O.bwt_aux(T, 1 << 10)
    assert codec.unbwt(U, T.size + 1)[0] == -1
    bad = I.copy()
    bad[2] = 0
    assert codec.unbwt_aux(U, 1 << 10, bad)[0] == -1


def _single_cycle(U, idx):
    """True when the LF walk from the sentinel row visits every row (a valid BWT)."""
    n = U.size
    L = np.concatenate([U[:idx], [0], U[idx:]]).astype(np.int64)
    cnt = np.bincount(U, minlength=256)
    base = 1 + np.concatenate([[0], np.cumsum(cnt)[:-1]])
    lf = np.zeros(n + 1, np.int64)
    seen = base.copy()
    for q in range(n + 1):
        if q == idx:
            continue
        c = L[q]
        lf[q] = seen[c]
        seen[c] += 1
    r, steps = 0, 0
    while True:
        r = lf[r] if r != idx else 0
        steps += 1
        if r == 0:
            break
    return steps == n + 1


def test_invalid_bwt_is_reported_valid_random_strings_decode():
    """Random strings: the ones whose LF permutation is one cycle decode exactly like the oracle; the others are
    not a BWT of any text with that primary index and are refused with -1."""
    rng = np.random.default_rng(3)
    nvalid = ninvalid = 0
    for it in range(300):
        n = int(rng.integers(2, 40))
        U = rng.integers(0, 3, n).astype(np.uint8)
        idx = int(rng.integers(1, n + 1))
        rc, back = codec.unbwt(U, idx)
        if _single_cycle(U, idx):
            nvalid += 1
            orc, oback = O.unbwt(U, idx)
            assert rc == 0 and np.array_equal(back, oback)
        else:
            ninvalid += 1
            assert rc == -1
    assert nvalid > 20 and ninvalid > 20


def test_inverse_large_blocks_round_trip():
    for T in (W.zipf_prose(16 << 20, 5), W.periodic(8 << 20, 2, 1, 1 << 20), W.fibonacci(4 << 20)):
        rc, U, I = codec.bwt_aux(T, 1 << 20)
        assert rc == 0
        rc, back = codec.unbwt_aux(U, 1 << 20, I)
        assert rc == 0 and np.array_equal(back, T)
