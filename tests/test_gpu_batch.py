"""Batched forward and inverse: many uneven blocks from the three mixed-batch sources in one device pass; every
block equals its single-block result and the oracle; the batched answer never depends on batch composition."""
import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec, native
from kolmo_gb300 import workloads as W
from kolmo_gb300.host import codec18_rlog

pytestmark = pytest.mark.gpu


def _mixed(count, lo, hi, seed):
    return [t for _, t in W.mixed_batch(count, lo, hi, seed)]


def test_batch_forward_equals_oracle_and_single_calls():
    blocks = _mixed(48, 16 << 10, 2 << 20, 17)
    jobs = [(t, 1 << codec18_rlog(t.size)) for t in blocks]
    rc, res = codec.fwd_batch(jobs)
    assert rc == 0, native.last_error()
    for (t, r), (brc, U, I) in zip(jobs, res):
        orc, oU, oI = O.bwt_aux(t, r)
        assert brc == 0 and np.array_equal(U, oU) and np.array_equal(I, oI)
    # a block's result does not depend on the batch it was sorted in
    for k in (0, 7, 31):
        rc1, U1, I1 = codec.bwt_aux(*jobs[k])
        assert rc1 == 0 and np.array_equal(U1, res[k][1]) and np.array_equal(I1, res[k][2])
    rc2, res2 = codec.fwd_batch(jobs[::-1], plain=True)
    assert rc2 == 0
    for a, b in zip(res, res2[::-1]):
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_batch_inverse_round_trip():
    blocks = _mixed(48, 16 << 10, 2 << 20, 18)
    jobs = [(t, 1 << codec18_rlog(t.size)) for t in blocks]
    rc, res = codec.fwd_batch(jobs)
    assert rc == 0
    rc, back = codec.inv_batch([(U, r, I) for (t, r), (_, U, I) in zip(jobs, res)])
    assert rc == 0, native.last_error()
    for t, (brc, b) in zip(blocks, back):
        assert brc == 0 and np.array_equal(b, t)


def test_batch_with_invalid_jobs_reports_per_job():
    t = W.markov2(10_000, 2)
    rc, res = codec.fwd_batch([(t, 1 << 10), (t, 3), (t[:1], 2), (t[:0], 2)])
    assert rc == -1
    assert [x[0] for x in res] == [0, -1, 0, 0]
    assert np.array_equal(res[0][1], O.bwt_aux(t, 1 << 10)[1])
