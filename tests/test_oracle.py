"""The CPU oracle (oracle/oracle.c) pinned against the reference: the golden vectors made by the reference's own
sorter, and -- where the reference sorter was built on this machine -- the reference itself, live. Also the
reference's argument checks and edge cases (tests/test_bwt.c:97-121)."""
import numpy as np
import pytest

import oracle as O
from golden_cases import h, make_input
from kolmo_gb300 import workloads as W
import refgen as R
from kolmo_gb300.host import codec18_rlog


def _small(c):
    return c["n"] <= 1_100_000


def test_oracle_matches_golden(golden):
    """Every golden case: U, I and the suffix array of the oracle equal the reference's (hashes)."""
    for c in golden:
        if not _small(c):
            continue
        T = make_input(c)
        assert h(T) == c["input"], f"{c['name']}: input generator drifted"
        rc, U, I, SA = O.bwt_aux(T, c["r"], want_sa=True)
        assert rc == 0
        assert h(U) == c["U"], c["name"]
        assert h(I.astype("<i4")) == c["I"], c["name"]
        assert int(I[0]) == c["I0"]
        assert h(SA.astype("<i4")) == c["SA"], c["name"]


def test_oracle_tiny_full_vectors(golden):
    for c in golden:
        if "U_hex" not in c:
            continue
        T = np.frombuffer(bytes.fromhex(c["T_hex"]), np.uint8)
        rc, U, I = O.bwt_aux(T, c["r"])
        assert rc == 0 and U.tobytes().hex() == c["U_hex"] and [int(x) for x in I] == c["I_list"]


def test_oracle_inverse_restores_golden_inputs(golden):
    for c in golden:
        if c["n"] > 300_000:
            continue
        T = make_input(c)
        rc, U, I = O.bwt_aux(T, c["r"])
        rc2, back = O.unbwt_aux(U, c["r"], I)
        assert rc2 == 0 and np.array_equal(back, T), c["name"]
        rc3, back2 = O.unbwt(U, int(I[0]))
        assert rc3 == 0 and np.array_equal(back2, T)


def test_suffix_array_is_sorted_naive():
    """Second check of the SA for small n: a comparison sort of the suffixes (implicit smallest sentinel)."""
    rng = np.random.default_rng(5)
    for n in (1, 2, 5, 50, 300):
        for alpha in (1, 2, 4, 256):
            T = rng.integers(0, alpha, n).astype(np.uint8)
            b = T.tobytes()
            ref = sorted(range(n), key=lambda i: b[i:])
            assert list(O.suffix_array(T)) == ref


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sorter not built on this machine")
def test_oracle_matches_reference_live():
    rng = np.random.default_rng(7)
    for it in range(40):
        n = int(rng.integers(2, 200_000))
        alpha = int(rng.integers(1, 257))
        T = rng.integers(0, alpha, n).astype(np.uint8)
        if it % 5 == 1 and n > 1000:
            for i in range(1000, n):
                if rng.integers(0, 1000):
                    T[i] = T[i - 997]
        for r in (2, 1 << 10, 1 << codec18_rlog(n)):
            a = O.bwt_aux(T, r)
            b = O.bwt_aux(T, r, use_ref=True)
            assert a[0] == b[0] == 0
            assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sorter not built on this machine")
def test_argument_checks_match_reference():
    T = R.test_block(1, 100)
    for r in (0, 1, 3, 6, -2):
        assert O.bwt_aux(T, r)[0] == -1 == O.bwt_aux(T, r, use_ref=True)[0]
    rc, U, I = O.bwt_aux(T, 4)
    bad = I.copy()
    bad[0] = 101
    assert O.unbwt_aux(U, 4, bad)[0] == -1 == O.unbwt_aux(U, 4, bad, use_ref=True)[0]
    bad[0] = 0
    assert O.unbwt_aux(U, 4, bad)[0] == -1 == O.unbwt_aux(U, 4, bad, use_ref=True)[0]
    assert O.unbwt(U, 101)[0] == -1 == O.unbwt(U, 101, use_ref=True)[0]
    for n in (0, 1):
        T = R.test_block(1, n)
        a, b = O.bwt_aux(T, 2), O.bwt_aux(T, 2, use_ref=True)
        assert a[0] == b[0] == 0 and np.array_equal(a[1], b[1]) and int(a[2][0]) == int(b[2][0]) == n


def test_planted_mistake_is_caught(golden):
    """A wrong oracle must fail the golden comparison: plant a byte swap in the oracle's output."""
    c = next(c for c in golden if c["name"] == "markov_1mib")
    T = make_input(c)
    rc, U, I = O.bwt_aux(T, c["r"])
    U2 = U.copy()
    U2[[10, 11]] = U2[[11, 10]]
    if U2[10] != U2[11]:
        assert h(U2) != c["U"]


@pytest.mark.parametrize("n,r", [(2, 2), (100, 8), (4097, 512), (300_000, 1 << 12), (1 << 20, 1 << 17)])
def test_threaded_decode_equals_serial(n, r):
    """The restatement's multi-threaded per-sample decode (the CPU baseline's inverse) equals the serial LF walk."""
    T = W.markov2(n, n % 1000 + 1)
    rc, U, I = O.bwt_aux(T, r)
    assert rc == 0
    for threads in (1, 3, 8):
        rc2, back = O.unbwt_aux(U, r, I, threads=threads)
        assert rc2 == 0 and np.array_equal(back, T)
    bad = I.copy()
    bad[-1] = n + 1
    assert O.unbwt_aux(U, r, bad, threads=4)[0] == -1
