"""Forward BWT on the GPU against the reference's outputs (golden hashes from the reference sorter) and the CPU
oracle. Bit-exact: U, the sampled indexes and the suffix array. Cases follow the reference's own tests
(tests/test_bwt.c:97-121 kinds and sizes; tests/test_gpu_sa.c:74-98 edge kinds and random inputs with repeats)."""
import ctypes
import os

import numpy as np
import pytest

import oracle as O
from golden_cases import h, make_input
from kolmo_gb300 import codec, native
from kolmo_gb300 import workloads as W
import refgen as R
from kolmo_gb300.host import codec18_rlog

pytestmark = pytest.mark.gpu


def test_forward_matches_reference_golden(golden):
    for c in golden:
        T = make_input(c)
        assert h(T) == c["input"], f"{c['name']}: input generator drifted on this machine"
        rc, U, I = codec.bwt_aux(T, c["r"])
        assert rc == 0, (c["name"], native.last_error())
        assert h(U) == c["U"], c["name"]
        assert h(I.astype("<i4")) == c["I"], c["name"]
        assert int(I[0]) == c["I0"]


def test_forward_tiny_full_vectors(golden):
    for c in golden:
        if "U_hex" in c:
            T = np.frombuffer(bytes.fromhex(c["T_hex"]), np.uint8)
            rc, U, I = codec.bwt_aux(T, c["r"])
            assert rc == 0 and U.tobytes().hex() == c["U_hex"] and [int(x) for x in I] == c["I_list"]


def _edge_inputs():
    """tests/test_gpu_sa.c:74-86: n = 2..299 for seven kinds (zeros, one letter, alternating, periodic, random
    binary, half zeros then ternary, random bytes)."""
    rng = np.random.default_rng(0x9E3779B9)
    out = []
    for n in range(2, 300):
        for kind in range(7):
            i = np.arange(n)
            if kind == 0:
                t = np.zeros(n, np.uint8)
            elif kind == 1:
                t = np.full(n, ord("a"), np.uint8)
            elif kind == 2:
                t = (i % 2).astype(np.uint8)
            elif kind == 3:
                t = np.frombuffer(b"abcab", np.uint8)[i % 5]
            elif kind == 4:
                t = rng.integers(0, 2, n).astype(np.uint8)
            elif kind == 5:
                t = np.where(i < n // 2, 0, rng.integers(0, 3, n)).astype(np.uint8)
            else:
                t = rng.integers(0, 256, n).astype(np.uint8)
            out.append(t)
    return out


def test_forward_edge_kinds_batched():
    """2086 small blocks in one batch: each equals the oracle (and the batch equals per-block answers)."""
    blocks = _edge_inputs()
    rc, res = codec.fwd_batch([(t, 2) for t in blocks])
    assert rc == 0, native.last_error()
    for t, (brc, U, I) in zip(blocks, res):
        orc, oU, oI = O.bwt_aux(t, 2)
        assert brc == 0 and np.array_equal(U, oU) and np.array_equal(I, oI), t.tobytes()[:40]


def test_forward_random_with_repeats():
    """tests/test_gpu_sa.c:87-98: 60 random inputs (small alphabets, copies of an earlier stretch), up to 3 MB."""
    rng = np.random.default_rng(60)
    for it in range(60):
        n = 2 + int(rng.integers(0, 70000 if it < 40 else 3000000))
        alpha = 1 + int(rng.integers(0, 3 if it % 4 == 0 else 256))
        t = rng.integers(0, alpha, n).astype(np.uint8)
        if it % 5 == 1 and n > 1000:
            keep = rng.integers(0, 1000, n - 1000) != 0
            idx = np.arange(1000, n)
            for i in idx[keep][:200000]:
                t[i] = t[i - 997]
        r = 1 << codec18_rlog(n)
        rc, U, I = codec.bwt_aux(t, r)
        orc, oU, oI = O.bwt_aux(t, r)
        assert rc == 0 and np.array_equal(U, oU) and np.array_equal(I, oI), (it, n, alpha)


def test_plain_path_equals_graph_path(golden):
    names = {"markov_1mib", "periodic/7/1048576", "fibonacci/1048576", "test_block/8/1000003/524288"}
    cases = [c for c in golden if c["name"] in names]
    assert cases
    blocks = [(make_input(c), c["r"]) for c in cases]
    rc1, a = codec.fwd_batch(blocks, plain=True)
    assert rc1 == 0
    for _ in range(2):  # a batch shape is captured as a graph the second time the graph path sees it
        rc2, b = codec.fwd_batch(blocks, plain=False)
        assert rc2 == 0
        for c, x, y in zip(cases, a, b):
            assert np.array_equal(x[1], y[1]) and np.array_equal(x[2], y[2])
            assert h(x[1]) == c["U"]


def test_in_place_T_equals_U():
    """T == U is allowed (sais.h:10): the caller's buffer is overwritten with the BWT."""
    T = W.markov2(100_000, 3)
    orc, oU, oI = O.bwt_aux(T, 1 << 13)
    buf = T.copy()
    I = np.zeros(16, np.int32)
    A = np.zeros(1, np.int32)
    rc = native.lib().kolmo_sais_bwt_aux(buf.ctypes.data, buf.ctypes.data, A.ctypes.data, buf.size, 1 << 13,
                                         I.ctypes.data, 4)
    assert rc == 0 and np.array_equal(buf, oU) and np.array_equal(I[: oI.size], oI)


def test_suffix_array_output_matches_oracle():
    import torch

    eng = codec.Engine()
    for T in (W.markov2(300_000, 5), W.periodic(200_000, 3, 7, 1 << 16), R.test_block(8, 250_000)):
        n = T.size
        dT = torch.zeros(n + 64, dtype=torch.uint8, device="cuda")
        dT[:n] = torch.from_numpy(T).cuda()
        dL = torch.zeros(n + 1, dtype=torch.uint8, device="cuda")
        dI = torch.zeros(8, dtype=torch.int32, device="cuda")
        dSA = torch.zeros(n, dtype=torch.int32, device="cuda")
        assert eng.fwd(dT, dL, dI, [(0, n, 1 << 16, 0)], dSA=dSA) == 0
        assert eng.wait()[0] == 0
        assert np.array_equal(dSA.cpu().numpy(), O.suffix_array(T))


def test_full_size_prose_round_trip_and_oracle():
    """The 64 MiB prose block: GPU forward equals the oracle; GPU inverse restores the text."""
    T = W.prose_64mib()
    r = 1 << codec18_rlog(T.size)
    rc, U, I = codec.bwt_aux(T, r)
    assert rc == 0, native.last_error()
    orc, oU, oI = O.bwt_aux(T, r)
    assert np.array_equal(I, oI) and np.array_equal(U, oU)
    rc, back = codec.unbwt_aux(U, r, I)
    assert rc == 0 and np.array_equal(back, T)


def _pin_forward(T, r, U, I):
    """Checks U and every sampled index of a large block: against the reference's own sorter where it was built on
    this machine (all host threads), else with the oracle's segment decoder, which decodes segment t of the text from
    I[t + 1] (a wrong sampled index corrupts its segment) and segment 0 from I[0]."""
    if O.ref_lib() is not None:
        rc, rU, rI = O.bwt_aux(T, r, use_ref=True, threads=os.cpu_count() or 1)
        assert rc == 0 and np.array_equal(I, rI), (I, rI)
        assert np.array_equal(U, rU)
    else:
        assert I.size > 1
        orc, back = O.unbwt_aux(U, r, I, threads=8)
        assert orc == 0 and np.array_equal(back, T)


def test_full_size_degenerate_blocks():
    """The 128 MiB degenerate inputs (periodic with periods 1, 7 and 4096 and one random flip per MiB; Fibonacci
    word): the GPU inverse restores the text from the GPU forward, and U with all its sampled indexes is pinned."""
    n = 128 << 20
    r = 1 << codec18_rlog(n)
    for kind in ("periodic-1", "periodic-7", "periodic-4096", "fibonacci"):
        T = W.degenerate(kind, n)
        rc, U, I = codec.bwt_aux(T, r)
        assert rc == 0, (kind, native.last_error())
        rc, back = codec.unbwt_aux(U, r, I)
        assert rc == 0 and np.array_equal(back, T), kind
        _pin_forward(T, r, U, I)


@pytest.mark.parametrize("mib", [24, 64])
def test_blocks_with_ranked_passes(mib):
    """Blocks of more than 16 M suffixes in a batch of at most 64 M write round 0's ranks in passes over id ranges
    (24 MiB: two passes, the last one partial; 64 MiB: four): the GPU inverse restores the text, and U with all its
    sampled indexes is pinned."""
    n = mib << 20
    T = W.zipf_prose(n, 600 + mib)
    r = 1 << codec18_rlog(n)
    rc, U, I = codec.bwt_aux(T, r)
    assert rc == 0, native.last_error()
    rc, back = codec.unbwt_aux(U, r, I)
    assert rc == 0 and np.array_equal(back, T)
    _pin_forward(T, r, U, I)
