"""The allocation-free inverse BWT (kgbwt_unbwt_noalloc), for callers that cannot allocate device memory: it must
decode exactly what the regular inverse entry point (kolmo_sais_unbwt_aux) decodes, on two calls in a row (its
static scratch keeps the previous call's contents), and refuse blocks above its fixed maximum.
This file is collected last so that a failure here never hides the results of the other tests."""
import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec, native
from kolmo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAX_N = 1 << 18


def _case(n, seed, r):
    T = W.markov2(n, seed)
    rc, U, I = O.bwt_aux(T, r)  # the BWT to decode (made by the CPU oracle)
    assert rc == 0
    return T, U, I


def test_no_alloc_inverse_matches_existing_entry_point():
    import torch

    lib = native.lib()
    cases = [(200_000, 41, 1 << 13), (MAX_N, 42, 1 << 15), (5_000, 43, 1 << 9)]
    for n, seed, r in cases:  # consecutive calls share the static scratch
        T, U, I = _case(n, seed, r)
        rc_ref, out_ref = codec.unbwt_aux(U, r, I)  # the existing inverse entry point
        assert rc_ref == 0 and np.array_equal(out_ref, T)
        dU = torch.from_numpy(U.copy()).cuda()
        dT = torch.zeros(n, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        rc = lib.kgbwt_unbwt_noalloc(dU.data_ptr(), dT.data_ptr(), n, int(I[0]), None)
        assert rc == 0, native.last_error()
        assert np.array_equal(dT.cpu().numpy(), out_ref)


def test_no_alloc_refuses_oversize_and_bad_arguments():
    import torch

    lib = native.lib()
    buf = torch.zeros(MAX_N + 64, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    assert lib.kgbwt_unbwt_noalloc(p, p, MAX_N + 1, 1, None) == -1
    assert "maximum" in native.last_error()
    assert lib.kgbwt_unbwt_noalloc(p, p, 100, 0, None) == -1
    assert lib.kgbwt_unbwt_noalloc(p, p, 100, 101, None) == -1
    assert lib.kgbwt_unbwt_noalloc(None, p, 100, 1, None) == -1
    host = np.zeros(1000, np.uint8)  # a host buffer is refused before any kernel sees it
    assert lib.kgbwt_unbwt_noalloc(host.ctypes.data, p, 1000, 1, None) == -1
    assert lib.kgbwt_unbwt_noalloc(p, host.ctypes.data, 1000, 1, None) == -1


def test_no_alloc_reports_an_invalid_string_and_stays_usable():
    """A string that is no BWT for its primary index returns -1 from the status word; the next valid call on the same
    static scratch still decodes like the existing entry point."""
    import torch

    lib = native.lib()
    n = 1000
    # 'a' * n with the sentinel in row 1: rows 0 and 1 form an LF cycle of their own
    dU = torch.full((n,), ord("a"), dtype=torch.uint8, device="cuda")
    dT = torch.zeros(n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert lib.kgbwt_unbwt_noalloc(dU.data_ptr(), dT.data_ptr(), n, 1, None) == -1
    assert "not a valid BWT" in native.last_error()
    T, U, I = _case(120_000, 44, 1 << 12)
    rc_ref, out_ref = codec.unbwt_aux(U, 1 << 12, I)
    assert rc_ref == 0
    dU = torch.from_numpy(U.copy()).cuda()
    dT = torch.zeros(U.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert lib.kgbwt_unbwt_noalloc(dU.data_ptr(), dT.data_ptr(), U.size, int(I[0]), None) == 0
    assert np.array_equal(dT.cpu().numpy(), out_ref)
