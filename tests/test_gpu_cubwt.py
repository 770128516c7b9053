"""libcubwt's entry points on the GPU (the path libbsc's GPU hook takes, reference src/arch/metal/cubwt_metal.c):
bwt_aux gives the drop-in call's (and the oracle's) bytes and indexes, bwt returns the primary index, unbwt restores
the text, and one storage serves calls of different sizes in a row."""
import ctypes

import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import native
from kolmo_gb300 import workloads as W
from test_gpu_inverse import _single_cycle

pytestmark = pytest.mark.gpu


def test_cubwt_matches_drop_in_and_oracle():
    lib = native.lib()
    st = ctypes.c_void_p()
    assert lib.libcubwt_allocate_device_storage(ctypes.byref(st), 4 << 20) == 0
    try:
        for n, r, seed in ((1 << 20, 1 << 17, 1), (300_001, 1 << 12, 2), (70_000, 1 << 16, 3), (4 << 20, 1 << 19, 4)):
            T = W.markov2(n, seed) if seed % 2 else W.zipf_prose(n, seed)
            L = np.zeros(n, np.uint8)
            I = np.zeros((n - 1) // r + 1, np.uint32)
            assert lib.libcubwt_bwt_aux(st, T.ctypes.data, L.ctypes.data, n, r, I.ctypes.data) == 0
            orc, oU, oI = O.bwt_aux(T, r)
            assert np.array_equal(L, oU) and np.array_equal(I.astype(np.int32), oI)
            L2 = np.zeros(n, np.uint8)
            p0 = lib.libcubwt_bwt(st, T.ctypes.data, L2.ctypes.data, n)
            assert p0 == int(oI[0]) and np.array_equal(L2, oU)
            back = np.zeros(n, np.uint8)
            assert lib.libcubwt_unbwt(st, L.ctypes.data, back.ctypes.data, n, None, int(I[0])) == 0
            assert np.array_equal(back, T)
        # a string that is not a valid BWT for its index (its LF permutation is not one cycle): an error, never a hang
        U = np.frombuffer(b"banana" * 1000, np.uint8).copy()
        assert not _single_cycle(U, 1)
        out = np.zeros(U.size, np.uint8)
        assert lib.libcubwt_unbwt(st, U.ctypes.data, out.ctypes.data, U.size, None, 1) < 0
    finally:
        assert lib.libcubwt_free_device_storage(st) == 0
