"""The request server's host logic without a GPU: the batching and admission policy (kgbwt_server_plan), the device
memory estimates it uses, and the request life cycle under injected device-allocation failures (the test hook makes
every batch fail with -2 before any device call), waits with timeouts, unknown ids and shutdown."""
import numpy as np
import pytest

from kolmo_gb300 import codec, native

FWD, INV = native.REQ_FWD, native.REQ_INV


def test_estimates_grow_with_size_and_batch():
    a = codec.estimate_bytes(FWD, [1 << 20], [1 << 17])
    b = codec.estimate_bytes(FWD, [4 << 20], [1 << 19])
    c = codec.estimate_bytes(FWD, [1 << 20, 1 << 20], [1 << 17, 1 << 17])
    assert 0 < a < b and a < c
    i = codec.estimate_bytes(INV, [1 << 20], [1 << 17])
    assert 0 < i < a  # the inverse needs far less than the forward sort
    assert codec.estimate_bytes(FWD, [1], [2]) == 0  # n <= 1 never touches the device


def test_plan_takes_oldest_kind_in_order():
    kinds = [INV, FWD, INV, INV, FWD, INV]
    sizes = [1000, 2000, 3000, 4000, 5000, 6000]
    rs = [1 << 8] * 6
    assert codec.server_plan(kinds, sizes, rs, 0, 0, 1 << 62) == [0, 2, 3, 5]
    assert codec.server_plan(kinds[1:], sizes[1:], rs[1:], 0, 0, 1 << 62) == [0, 3]


def test_plan_respects_budget_and_batch_bytes():
    sizes = [1 << 20] * 8
    rs = [1 << 17] * 8
    kinds = [FWD] * 8
    one = codec.estimate_bytes(FWD, sizes[:1], rs[:1])
    three = codec.estimate_bytes(FWD, sizes[:3], rs[:3])
    four = codec.estimate_bytes(FWD, sizes[:4], rs[:4])
    assert codec.server_plan(kinds, sizes, rs, 0, 0, three) == [0, 1, 2]
    assert codec.server_plan(kinds, sizes, rs, 0, 0, four - 1) == [0, 1, 2]
    assert codec.server_plan(kinds, sizes, rs, 0, 0, one - 1) == []           # the oldest does not fit
    assert codec.server_plan(kinds, sizes, rs, 0, 0, 1 << 62, 3 << 20) == [0, 1, 2]  # input bytes cap
    assert codec.server_plan(kinds, sizes, rs, 0, 0, 1 << 62, 1) == [0]       # the first is exempt from the cap
    # a worker that already holds a large forward workspace needs nothing more for a small batch
    assert codec.server_plan(kinds, sizes, rs, four, 0, four) == [0, 1, 2, 3]


def test_plan_stops_at_first_request_of_the_kind_that_does_not_fit():
    kinds = [FWD, FWD, INV, FWD]
    sizes = [1 << 16, 8 << 20, 1 << 16, 1 << 16]
    rs = [1 << 13, 1 << 20, 1 << 13, 1 << 13]
    small = codec.estimate_bytes(FWD, [1 << 16, 1 << 16], [1 << 13, 1 << 13])
    assert codec.server_plan(kinds, sizes, rs, 0, 0, small) == [0]  # request 3 must not overtake request 1


def test_injected_allocation_failures_fail_requests_not_the_server():
    srv = codec.Server(slots=2)
    try:
        assert srv.inject_oom(1000) == 0
        rng = np.random.default_rng(1)
        ids = []
        for k in range(12):
            T = rng.integers(0, 256, 5000 + 100 * k, dtype=np.uint8)
            if k % 3:
                ids.append(srv.submit_fwd(T, 1 << 8)[0])
            else:
                I = np.array([1] + [1] * ((T.size - 1) >> 8), np.int32)
                ids.append(srv.submit_inv(T, 1 << 8, I)[0])
        for rid in ids:
            st, rc, lat = srv.wait(rid, 20000)
            assert st == 1 and rc == -2 and lat >= 0
        s = srv.stats()
        assert s["submitted"] == 12 and s["failed"] == 12 and s["completed"] == 0 and s["batches"] >= 1
        assert srv.wait(ids[0], 0)[0] == -1  # forgotten once waited
        assert srv.cancel(12345) == -1
    finally:
        srv.close()


def test_bad_requests_are_refused_at_submission():
    srv = codec.Server(slots=1)
    try:
        T = np.zeros(100, np.uint8)
        with pytest.raises(ValueError):
            srv.submit_fwd(T, 3)  # not a power of two
        with pytest.raises(ValueError):
            srv.submit_inv(T, 5, np.ones(1, np.int32))
    finally:
        srv.close()
