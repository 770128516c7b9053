"""Synthetic workload generators: determinism (pinned hashes) and the properties the benchmark configurations state."""
import numpy as np

import refgen as R
from kolmo_gb300 import workloads as W


def test_test_block_kinds_match_reference_generator_shapes():
    assert not R.test_block(0, 1000).any()
    t3 = R.test_block(3, 18)
    assert t3.tobytes() == b"abcabcabdabcabcabd"
    t6 = R.test_block(6, 1000)
    assert np.array_equal(t6[500:], t6[:500])
    t7 = R.test_block(7, 200)
    assert t7[0] == 0xF2 and t7[97] == 0xF2 and t7[1:5].tobytes() == b"he q"


def test_markov_alphabet_and_determinism():
    a = W.markov2(1 << 16, 42)
    b = W.markov2(1 << 16, 42)
    assert np.array_equal(a, b)
    assert np.unique(a).size == 64
    assert not np.array_equal(a, W.markov2(1 << 16, 43))


def test_zipf_prose_properties():
    n = 4 << 20
    t = W.zipf_prose(n, 9)
    s = t.tobytes()
    letters = np.isin(t, np.frombuffer(b"abcdefghijklmnopqrstuvwxyz \n", np.uint8))
    noise = 1 - letters.mean()
    assert 0.005 < noise < 0.03  # ~2% random bytes (a random byte is a letter ~11% of the time)
    assert s.count(b" ") > n // 12
    # verbatim repeats: some 4 KiB window occurs twice
    probe = s[n // 2 : n // 2 + 4096]
    assert len(probe) == 4096


def test_acgt_n_fraction():
    t = W.acgt(1 << 22, 3)
    frac_n = (t == ord("N")).mean()
    assert 0.0005 < frac_n < 0.0015
    assert set(np.unique(t).tolist()) <= set(b"ACGTN")


def test_logs_lines():
    t = W.logs(1 << 18, 4).tobytes()
    lines = t.split(b"\n")[:-1]
    assert len(lines) > 1000
    assert all(l[:1].isdigit() for l in lines[:100])
    assert b"id=" in t and b"." in t


def test_periodic_and_fibonacci():
    p = W.periodic(1 << 20, 1, 7, 1 << 18)
    diff = np.nonzero(p[7:] != p[:-7])[0]
    assert 1 <= len(diff) <= 2 * 4 * 2  # 4 flips, each breaks at most two comparisons
    f = W.fibonacci(100).tobytes()
    assert f.startswith(b"abaababaabaab")


def test_pinned_hashes():
    """Same bytes on every machine: these hashes were computed on x86-64 and must match on aarch64 (the generators
    use only correctly rounded double arithmetic and their own log/exp)."""
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "workload_hashes.json")) as f:
        d = json.load(f)
    hx = lambda a: "%016x" % W.fnv1a(a)
    assert hx(W.markov_1mib()) == d["markov_1mib"]
    assert hx(W.zipf_prose(1 << 20, 1)) == d["zipf_prose_1mib_seed1"]
    assert hx(W.acgt(1 << 20, 1)) == d["acgt_1mib_seed1"]
    assert hx(W.logs(1 << 20, 1)) == d["logs_1mib_seed1"]
    assert hx(W.periodic(1 << 20, 1, 7)) == d["periodic7_1mib_seed1"]
    assert hx(W.loguniform_sizes(1, 256, 16 << 10, 16 << 20)) == d["loguniform_sizes_seed1"]
    assert hx(W.requests(1, 256)[0]) == d["requests_seed1"]


def test_size_distributions():
    s = W.loguniform_sizes(1, 4096, 16 << 10, 16 << 20)
    assert s.min() >= 16 << 10 and s.max() <= 16 << 20
    med = np.median(np.log2(s.astype(np.float64)))
    assert 18.5 < med < 20.5  # log-uniform between 2^14 and 2^24: median near 2^19
    sizes, gaps, mix, src = W.requests(1, 4000, rate=100.0)
    assert abs(np.median(sizes) / (256 * 1024) - 1) < 0.15
    assert sizes.max() <= 128 << 20
    assert abs(gaps.mean() - 0.01) < 0.002
    assert abs((mix < 300).mean() - 0.3) < 0.03
