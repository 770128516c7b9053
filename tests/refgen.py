"""Test infrastructure: the reference's suffix-sorter test blocks (tests/refgen.c, the generator of the reference's
tests/test_bwt.c:24-45), compiled on first use into tests/_build/ and loaded with ctypes."""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "refgen.c")
LIB = os.path.join(HERE, "_build", "librefgen.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
            os.makedirs(os.path.dirname(LIB), exist_ok=True)
            fd, tmp = tempfile.mkstemp(suffix=".so", dir=os.path.dirname(LIB))
            os.close(fd)
            subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp, SRC], check=True)
            os.replace(tmp, LIB)  # atomic: concurrent test processes never load a half-written library
        L = ctypes.CDLL(LIB)
        L.kgw_test_block.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.kgw_test_block.restype = None
        _lib = L
    return _lib


def test_block(kind: int, n: int) -> np.ndarray:
    """Block `kind` (0-8) of n bytes of the reference's suffix-sorter tests."""
    out = np.empty(max(n, 1), np.uint8)
    lib().kgw_test_block(kind, n, out.ctypes.data)
    return out[:n]
