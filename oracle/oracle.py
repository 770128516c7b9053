"""ORACLE -- test infrastructure only: ctypes bindings for the CPU oracle of the GPU BWT path.

Two libraries live here, both built by ``oracle/Makefile``:

* ``liboracle.so`` -- the C restatement in ``oracle.c`` (SA-IS plus the reference's BWT conventions and the LF-walk
  inverse; see that file's header for the reference lines each function follows).
* ``_ref/libkref.so`` -- the reference's own sorter, compiled from its ``src/algo/sais/sais.c`` and
  ``src/algo/par.c`` when the reference tree is present on the machine that built it.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_P = ctypes.c_void_p
_I32 = ctypes.c_int32


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class _Lib:
    def __init__(self, path: str, prefix: str):
        self.path = path
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix


_port = None
_ref = None


def port_lib():
    """The C restatement (always built)."""
    global _port
    if _port is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError(f"oracle not built: {path} (run make -C oracle)")
        lib = ctypes.CDLL(path)
        for name in ("orc_bwt_aux", "orc_unbwt_aux", "orc_unbwt", "orc_sa", "orc_sa_from_bwt", "orc_bwt_aux_sa"):
            getattr(lib, name).restype = _I32
        lib.orc_bwt_aux.argtypes = [_P, _P, _P, _I32, _I32, _P]
        lib.orc_bwt_aux_sa.argtypes = [_P, _P, _P, _I32, _I32, _P, _P]
        lib.orc_unbwt_aux.argtypes = [_P, _P, _P, _I32, _I32, _P]
        lib.orc_unbwt_aux_mt.argtypes = [_P, _P, _P, _I32, _I32, _P, _I32]
        lib.orc_unbwt_aux_mt.restype = _I32
        lib.orc_unbwt.argtypes = [_P, _P, _P, _I32, _I32]
        lib.orc_sa.argtypes = [_P, _P, _I32]
        lib.orc_sa_from_bwt.argtypes = [_P, _I32, _I32, _P]
        lib.orc_fnv1a.restype = ctypes.c_uint64
        lib.orc_fnv1a.argtypes = [_P, ctypes.c_uint64]
        _port = lib
    return _port


def ref_lib():
    """The reference's own sorter, or None when it was not built on this machine (or cannot load here)."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libkref.so")
        if not os.path.exists(path):
            return None
        try:
            lib = ctypes.CDLL(path)
        except OSError:
            return None
        lib.kolmo_sais_bwt_aux.restype = _I32
        lib.kolmo_sais_bwt_aux.argtypes = [_P, _P, _P, _I32, _I32, _P, _I32]
        lib.kolmo_sais_unbwt_aux.restype = _I32
        lib.kolmo_sais_unbwt_aux.argtypes = [_P, _P, _P, _I32, _I32, _P, _I32]
        lib.kolmo_sais_unbwt.restype = _I32
        lib.kolmo_sais_unbwt.argtypes = [_P, _P, _P, _I32, _I32, _I32]
        _ref = lib
    return _ref


def n_samples(n: int, r: int) -> int:
    return (n - 1) // r + 1 if n > 0 and r > 0 else 1


def bwt_aux(T: np.ndarray, r: int, use_ref: bool = False, threads: int = 1, want_sa: bool = False):
    """Forward BWT: returns (rc, U, I[, SA]) with the reference's conventions."""
    n = int(T.size)
    U = np.zeros(max(n, 1), np.uint8)
    A = np.zeros(n + 1, np.int32)
    I = np.zeros(max(n_samples(n, r), 1) + 1, np.int32)
    SA = np.zeros(max(n, 1), np.int32) if want_sa else None
    Tc = np.ascontiguousarray(T, dtype=np.uint8)
    if use_ref:
        lib = ref_lib()
        if lib is None:
            raise RuntimeError("reference sorter not built on this machine")
        rc = lib.kolmo_sais_bwt_aux(_ptr(Tc), _ptr(U), _ptr(A), n, r, _ptr(I), threads)
        if want_sa and rc == 0:
            SA = sa_from_bwt(U[:n], int(I[0])) if n > 1 else np.zeros(n, np.int32)
    elif want_sa:
        rc = port_lib().orc_bwt_aux_sa(_ptr(Tc), _ptr(U), _ptr(A), n, r, _ptr(I), _ptr(SA))
    else:
        rc = port_lib().orc_bwt_aux(_ptr(Tc), _ptr(U), _ptr(A), n, r, _ptr(I))
    out = (int(rc), U[:n], I[: n_samples(n, r)])
    return out + ((SA[:n] if SA is not None else None),) if want_sa else out


def unbwt_aux(U: np.ndarray, r: int, I: np.ndarray, use_ref: bool = False, threads: int = 1):
    n = int(U.size)
    out = np.zeros(max(n, 1), np.uint8)
    A = np.zeros(n + 2, np.int32)
    Ic = np.ascontiguousarray(I, dtype=np.int32)
    Uc = np.ascontiguousarray(U, dtype=np.uint8)
    if use_ref:
        rc = ref_lib().kolmo_sais_unbwt_aux(_ptr(Uc), _ptr(out), _ptr(A), n, r, _ptr(Ic), threads)
    else:
        rc = (port_lib().orc_unbwt_aux_mt(_ptr(Uc), _ptr(out), _ptr(A), n, r, _ptr(Ic), threads) if threads > 1
              else port_lib().orc_unbwt_aux(_ptr(Uc), _ptr(out), _ptr(A), n, r, _ptr(Ic)))
    return int(rc), out[:n]


def unbwt(U: np.ndarray, idx: int, use_ref: bool = False, threads: int = 1):
    n = int(U.size)
    out = np.zeros(max(n, 1), np.uint8)
    A = np.zeros(n + 2, np.int32)
    Uc = np.ascontiguousarray(U, dtype=np.uint8)
    if use_ref:
        rc = ref_lib().kolmo_sais_unbwt(_ptr(Uc), _ptr(out), _ptr(A), n, idx, threads)
    else:
        rc = port_lib().orc_unbwt(_ptr(Uc), _ptr(out), _ptr(A), n, idx)
    return int(rc), out[:n]


def suffix_array(T: np.ndarray) -> np.ndarray:
    n = int(T.size)
    SA = np.zeros(max(n, 1), np.int32)
    Tc = np.ascontiguousarray(T, dtype=np.uint8)
    rc = port_lib().orc_sa(_ptr(Tc), _ptr(SA), n)
    if rc:
        raise RuntimeError(f"orc_sa failed: {rc}")
    return SA[:n]


def sa_from_bwt(U: np.ndarray, idx: int) -> np.ndarray:
    n = int(U.size)
    SA = np.zeros(max(n, 1), np.int32)
    Uc = np.ascontiguousarray(U, dtype=np.uint8)
    rc = port_lib().orc_sa_from_bwt(_ptr(Uc), n, idx, _ptr(SA))
    if rc:
        raise RuntimeError(f"orc_sa_from_bwt failed: {rc}")
    return SA[:n]


def fnv1a(b) -> int:
    a = np.ascontiguousarray(np.frombuffer(memoryview(b).cast("B"), np.uint8) if not isinstance(b, np.ndarray)
                             else b.view(np.uint8).ravel())
    return int(port_lib().orc_fnv1a(_ptr(a), a.size))
