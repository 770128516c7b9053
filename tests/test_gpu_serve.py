"""The request server on the GPU: every request's result in a mixed, concurrently submitted stream is the same as the
drop-in call's on that request alone (and the oracle's); pending requests can be cancelled; a tight HBM budget
serializes work without exceeding it; an injected allocation failure fails one batch and the server carries on."""
import threading

import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec, native
from kolmo_gb300 import workloads as W
from kolmo_gb300.host import codec18_rlog

pytestmark = pytest.mark.gpu


def _requests(count, seed):
    """(kind, text) pairs: lognormal sizes (median 48 KiB, capped at 2 MiB) from the three batch sources."""
    sizes, _gaps, mix, src = W.requests(seed, count, median=48 * 1024, sigma=1.5, cap=2 << 20)
    out = []
    for i in range(count):
        n = max(int(sizes[i]), 2)
        out.append(("fwd" if mix[i] < 300 else "inv", W.source_block(int(src[i]), n, seed + i)))
    return out


def test_mixed_stream_equals_results_alone():
    reqs = _requests(48, 71)
    alone = []
    for kind, T in reqs:  # the drop-in calls, one request at a time
        r = 1 << codec18_rlog(T.size)
        rc, U, I = codec.bwt_aux(T, r)
        assert rc == 0
        alone.append((r, U, I))
    srv = codec.Server(slots=3, hbm_budget=40 << 30)
    try:
        handles = [None] * len(reqs)

        def submit(lo):
            for i in range(lo, len(reqs), 2):
                kind, T = reqs[i]
                r, U, I = alone[i]
                handles[i] = (kind, srv.submit_fwd(T, r) if kind == "fwd" else srv.submit_inv(U, r, I))

        ths = [threading.Thread(target=submit, args=(k,)) for k in range(2)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        for i, (kind, h) in enumerate(handles):
            st, rc, lat = srv.wait(h[0], 120000)
            assert st == 1 and rc == 0, (i, kind, rc, native.last_error())
            T = reqs[i][1]
            r, U, I = alone[i]
            if kind == "fwd":
                assert np.array_equal(h[1], U) and np.array_equal(h[2], I), i
            else:
                assert np.array_equal(h[1], T), i
        s = srv.stats()
        assert s["completed"] == len(reqs) and s["failed"] == 0
        assert s["batches"] < len(reqs)  # requests were batched together
    finally:
        srv.close()
    # one forward result against the oracle as well
    i = next(k for k, (kind, _) in enumerate(reqs) if kind == "fwd")
    orc, oU, oI = O.bwt_aux(reqs[i][1], alone[i][0])
    assert np.array_equal(alone[i][1], oU) and np.array_equal(alone[i][2], oI)


def test_cancel_pending_requests():
    srv = codec.Server(slots=1)
    try:
        big = W.zipf_prose(16 << 20, 5)
        first = srv.submit_fwd(big, 1 << 21)
        small = [srv.submit_fwd(W.markov2(20000 + k, k), 1 << 12) for k in range(6)]
        cancelled = [h[0] for h in small[::2] if srv.cancel(h[0]) == 0]
        assert srv.wait(first[0], 120000)[:2] == (1, 0)
        for h in small:
            st, rc, _ = srv.wait(h[0], 120000)
            assert st == 1 and rc == (-3 if h[0] in cancelled else 0)
        assert srv.stats()["cancelled"] == len(cancelled)
    finally:
        srv.close()


def test_tight_budget_serializes_within_budget():
    texts = [W.markov2(3 << 20, 90 + k) for k in range(6)]
    r = 1 << codec18_rlog(texts[0].size)
    one = codec.estimate_bytes(native.REQ_FWD, [texts[0].size], [r])
    budget = int(one * 1.5)  # room for one request at a time
    srv = codec.Server(slots=3, hbm_budget=budget)
    try:
        hs = [srv.submit_fwd(T, r) for T in texts]
        for T, h in zip(texts, hs):
            assert srv.wait(h[0], 120000)[:2] == (1, 0)
            rc, U, I = codec.bwt_aux(T, r)
            assert np.array_equal(h[1], U) and np.array_equal(h[2], I)
        s = srv.stats()
        assert 0 < s["hbm_peak"] <= budget
        # a request that cannot fit the budget even alone fails with -2
        huge = W.markov2(32 << 20, 3)
        h = srv.submit_fwd(huge, 1 << 22)
        assert srv.wait(h[0], 120000)[:2] == (1, -2)
    finally:
        srv.close()


def test_injected_failure_then_recovery():
    srv = codec.Server(slots=1)
    try:
        T = W.markov2(200_000, 9)
        r = 1 << 15
        srv.inject_oom(1)
        h1 = srv.submit_fwd(T, r)
        assert srv.wait(h1[0], 120000)[:2] == (1, -2)
        h2 = srv.submit_fwd(T, r)
        assert srv.wait(h2[0], 120000)[:2] == (1, 0)
        rc, U, I = codec.bwt_aux(T, r)
        assert np.array_equal(h2[1], U) and np.array_equal(h2[2], I)
    finally:
        srv.close()
