"""The C-ABI library (no GPU needed): it loads, exports every function the public headers declare, and applies the
reference's argument checks before touching the device (src/algo/sais/sais.c:12029-12038, 12057-12068)."""
import ctypes
import os
import re

import numpy as np
import pytest

from kolmo_gb300 import build, codec, host, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    """Every function the public headers (include/kgbwt.h, include/kgbwt_cubwt.h) declare."""
    names = set()
    for h in ("kgbwt.h", "kgbwt_cubwt.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b((?:kolmo|kgbwt|libcubwt)_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(build.LIB):
        build.build_cuda()
    return native.lib()


def test_exports_every_declared_symbol(lib):
    names = _header_functions()
    assert "kolmo_sais_bwt_aux" in names and "kgbwt_engine_fwd" in names
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(native.EXPORTS) == names


def test_checked_build_exports_the_same(lib):
    if not os.path.exists(build.LIB_CHECKED):
        build.build_cuda(checked=True)
    chk = ctypes.CDLL(build.LIB_CHECKED)
    for name in _header_functions():
        assert hasattr(chk, name), name


def test_version(lib):
    assert lib.kgbwt_version() >= 100


def test_forward_argument_checks_without_device(lib):
    T = np.frombuffer(b"banana", np.uint8).copy()
    U = np.zeros(6, np.uint8)
    I = np.zeros(8, np.int32)
    A = np.zeros(8, np.int32)
    f = lib.kolmo_sais_bwt_aux
    assert f(None, U.ctypes.data, A.ctypes.data, 6, 2, I.ctypes.data, 1) == -1
    assert f(T.ctypes.data, None, A.ctypes.data, 6, 2, I.ctypes.data, 1) == -1
    assert f(T.ctypes.data, U.ctypes.data, None, 6, 2, I.ctypes.data, 1) == -1
    assert f(T.ctypes.data, U.ctypes.data, A.ctypes.data, 6, 2, None, 1) == -1
    assert f(T.ctypes.data, U.ctypes.data, A.ctypes.data, -1, 2, I.ctypes.data, 1) == -1
    for r in (0, 1, 3, 6, 12, -4):
        assert f(T.ctypes.data, U.ctypes.data, A.ctypes.data, 6, r, I.ctypes.data, 1) == -1
    # n <= 1: handled on the host exactly as the reference (U[0] = T[0], I[0] = n)
    assert f(T.ctypes.data, U.ctypes.data, A.ctypes.data, 1, 2, I.ctypes.data, 1) == 0
    assert U[0] == ord("b") and I[0] == 1
    assert f(T.ctypes.data, U.ctypes.data, A.ctypes.data, 0, 2, I.ctypes.data, 1) == 0 and I[0] == 0


def test_inverse_argument_checks_without_device(lib):
    U = np.frombuffer(b"annbaa", np.uint8).copy()
    out = np.zeros(6, np.uint8)
    A = np.zeros(8, np.int32)
    I = np.array([4, 1, 1, 1], np.int32)
    f = lib.kolmo_sais_unbwt_aux
    assert f(None, out.ctypes.data, A.ctypes.data, 6, 2, I.ctypes.data, 1) == -1
    assert f(U.ctypes.data, out.ctypes.data, None, 6, 2, I.ctypes.data, 1) == -1
    assert f(U.ctypes.data, out.ctypes.data, A.ctypes.data, 6, 3, I.ctypes.data, 1) == -1
    for bad in (0, 7, -1):
        J = I.copy()
        J[1] = bad
        assert f(U.ctypes.data, out.ctypes.data, A.ctypes.data, 6, 2, J.ctypes.data, 1) == -1
    assert lib.kolmo_sais_unbwt(U.ctypes.data, out.ctypes.data, A.ctypes.data, 6, 7, 1) == -1
    assert lib.kolmo_sais_unbwt(U.ctypes.data, out.ctypes.data, A.ctypes.data, 6, 0, 1) == -1
    # n <= 1
    J = np.array([1], np.int32)
    assert f(U.ctypes.data, out.ctypes.data, A.ctypes.data, 1, 1, J.ctypes.data, 1) == 0 and out[0] == U[0]
    J[0] = 0
    assert f(U.ctypes.data, out.ctypes.data, A.ctypes.data, 1, 1, J.ctypes.data, 1) == -1


def test_engine_argument_checks_without_device(lib):
    e = lib.kgbwt_engine_create()
    assert e
    assert lib.kgbwt_engine_config(e, 1000, 0, 0) == -1
    assert lib.kgbwt_engine_config(e, 8192, 1, 4) == 0
    blk = (native.Block * 1)(native.Block(0, 1, 2, 0))
    assert lib.kgbwt_engine_fwd(e, None, None, None, None, blk, 1, None, 0) == -1
    buf = np.zeros(64, np.uint8)
    ptr = buf.ctypes.data
    assert lib.kgbwt_engine_fwd(e, ptr + 1, ptr, ptr, None, blk, 1, None, 0) == -1  # unaligned text
    assert lib.kgbwt_engine_fwd(e, ptr, ptr, ptr, None, blk, 1, None, 0) == -1      # n < 2
    ib = (native.IBlock * 1)(native.IBlock(0, 8, 9, 0))
    assert lib.kgbwt_engine_inv(e, ptr, ptr, ib, 1, None, 0) == -1                  # p0 > n
    lib.kgbwt_engine_destroy(e)


def test_codec18_sampling_rule():
    """bwt_stream.c:224-227: r = largest power of two <= lz/8 (>= 2), at most 255 samples after I[0]."""
    assert host.codec18_rlog(1 << 20) == 17 and (((1 << 20) - 1) >> 17) == 7
    assert host.codec18_rlog(128 << 20) == 24
    for lz in (2, 3, 15, 16, 17, 1000, 65535, 65536, 1 << 24, (1 << 31) - 1):
        rl = host.codec18_rlog(lz)
        assert 1 <= rl <= 30 and ((lz - 1) >> rl) <= 255
    assert host.codec18_rlog(1 << 20, index_log2=3) == 12  # forced small interval raised to keep k <= 255
    assert host.codec5_r(1 << 20) == 1 << 17 and host.codec5_r(100) == 8


def test_python_mirror_checks_arguments(lib):
    assert codec.bwt_aux(np.zeros(10, np.uint8), 3)[0] == -1
    assert codec.unbwt(np.zeros(10, np.uint8), 0)[0] == -1


def test_cubwt_argument_checks_need_no_device(lib):
    """libcubwt's entry points refuse bad arguments before touching the device."""
    st = ctypes.c_void_p()
    assert lib.libcubwt_allocate_device_storage(ctypes.byref(st), -1) < 0
    assert lib.libcubwt_allocate_device_storage(ctypes.byref(st), 1 << 20) == 0 and st.value
    T = np.zeros(64, np.uint8)
    L = np.zeros(64, np.uint8)
    I = np.zeros(8, np.uint32)
    assert lib.libcubwt_bwt_aux(st, T.ctypes.data, L.ctypes.data, 1, 2, I.ctypes.data) < 0      # n < 2
    assert lib.libcubwt_bwt_aux(st, T.ctypes.data, L.ctypes.data, 64, 3, I.ctypes.data) < 0     # r not 2^k
    assert lib.libcubwt_bwt_aux(st, T.ctypes.data, L.ctypes.data, 64, 128, I.ctypes.data) < 0   # r > n
    assert lib.libcubwt_bwt_aux(None, T.ctypes.data, L.ctypes.data, 64, 8, I.ctypes.data) < 0   # no storage
    assert lib.libcubwt_unbwt(st, T.ctypes.data, L.ctypes.data, 64, None, 0) < 0                # i out of range
    assert lib.libcubwt_free_device_storage(st) == 0
