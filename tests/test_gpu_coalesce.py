"""Concurrent drop-in calls: the reference's block workers call the sorter from one thread per block
(src/core/blocks.c:181, src/core/compress.c:221, src/core/decode.c:405). Calls that arrive while the device worker is
busy are coalesced into one batch, and each call still gets the bytes it would get alone (the oracle's)."""
import os
import subprocess
import sys
import threading

import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec
from kolmo_gb300 import workloads as W
from kolmo_gb300.host import codec18_rlog

pytestmark = pytest.mark.gpu


def _blocks():
    out = []
    for i in range(12):
        n = (1 << 20) + 4099 * i
        T = W.markov2(n, 700 + i) if i % 3 == 0 else (W.zipf_prose(n, 800 + i) if i % 3 == 1 else W.acgt(n, 900 + i))
        out.append((T, 1 << codec18_rlog(n)))
    return out


def _concurrently(fn, args):
    res = [None] * len(args)
    gate = threading.Barrier(len(args))

    def work(i):
        gate.wait()
        res[i] = fn(*args[i])

    th = [threading.Thread(target=work, args=(i,)) for i in range(len(args))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return res


def test_concurrent_calls_coalesce_and_match_the_oracle():
    blocks = _blocks()
    want = [O.bwt_aux(T, r) for T, r in blocks]
    for _ in range(2):  # the second time the workspace exists already and the calls pile up behind a short batch
        before = codec.dropin_stats()
        got = _concurrently(codec.bwt_aux, blocks)
        after = codec.dropin_stats()
        for (T, r), (rc, U, I), (orc, oU, oI) in zip(blocks, got, want):
            assert rc == 0 and orc == 0
            assert np.array_equal(U, oU) and np.array_equal(I, oI), T.size
        calls = after["fwd_calls"] - before["fwd_calls"]
        batches = after["fwd_batches"] - before["fwd_batches"]
        assert calls == len(blocks) and 1 <= batches < calls, (calls, batches)
        before = codec.dropin_stats()
        back = _concurrently(codec.unbwt_aux, [(U, r, I) for (_, r), (_, U, I) in zip(blocks, got)])
        after = codec.dropin_stats()
        for (T, _), (rc, B) in zip(blocks, back):
            assert rc == 0 and np.array_equal(B, T)
        calls = after["inv_calls"] - before["inv_calls"]
        batches = after["inv_batches"] - before["inv_batches"]
        assert calls == len(blocks) and 1 <= batches < calls, (calls, batches)
    assert codec.dropin_stats()["retried"] == 0


def test_concurrent_calls_keep_their_own_return_codes():
    """Bad arguments and invalid BWT strings in a coalesced batch fail alone; their neighbours succeed."""
    T, r = W.markov2(300_000, 17), 1 << 15
    rc, U, I = codec.bwt_aux(T, r)
    assert rc == 0
    # 'a' * n with the sentinel in row 1: rows 0 and 1 form an LF cycle of their own, so it is no BWT string
    Ua = np.full(1000, ord("a"), np.uint8)
    args = [(U, r, I), (Ua, Ua.size, np.array([1], np.int32)), (U, r, I), (U, 3, I)]
    res = _concurrently(codec.unbwt_aux, args)
    assert res[0][0] == 0 and np.array_equal(res[0][1], T)
    assert res[2][0] == 0 and np.array_equal(res[2][1], T)
    assert res[1][0] == -1 and res[3][0] == -1


_CAPPED = r"""
import sys, threading
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/oracle")
import oracle as O
from kolmo_gb300 import codec
from kolmo_gb300 import workloads as W
blocks = [W.markov2(1 << 20, 300 + i) for i in range(8)]
want = [O.bwt_aux(T, 1 << 17) for T in blocks]
codec.bwt_aux(blocks[0], 1 << 17)  # the workspace exists: the timed calls queue behind short batches
gate = threading.Barrier(len(blocks)); res = [None] * len(blocks)
def work(i):
    gate.wait(); res[i] = codec.bwt_aux(blocks[i], 1 << 17)
th = [threading.Thread(target=work, args=(i,)) for i in range(len(blocks))]
[t.start() for t in th]; [t.join() for t in th]
for (rc, U, I), (orc, oU, oI) in zip(res, want):
    assert rc == 0 and np.array_equal(U, oU) and np.array_equal(I, oI)
st = codec.dropin_stats()
print(st["fwd_calls"], st["fwd_batches"], st["fwd_largest"])
"""


def test_batch_cap_bounds_coalesced_batches():
    """KGBWT_BATCH_MIB caps a coalesced batch's input: with a 2 MiB cap, concurrent 1 MiB calls are batched at most
    two at a time, and every call still gets the oracle's bytes (a fresh process, so the cap applies from its first
    call)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, KGBWT_BATCH_MIB="2")
    r = subprocess.run([sys.executable, "-c", _CAPPED, root], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    calls, batches, largest = (int(x) for x in r.stdout.split()[-3:])
    assert calls == 9 and 1 <= largest <= 2 and batches >= 5, (calls, batches, largest)
