"""ctypes bindings to ``libkgbwt.so``, the C ABI of the GPU block-sorting engine (``include/kgbwt.h``).

The library is loaded from the package's ``_native`` directory (built in-tree by ``kolmo_gb300.build``). There is no
CPU fallback: if the library is missing or cannot load, every call raises.
Set ``KGBWT_CHECKED=1`` to load the bounds-checked build instead (same ABI; device writes are range-checked).
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_U32 = ctypes.c_uint32


class FwdJob(ctypes.Structure):
    _fields_ = [("T", _P), ("U", _P), ("n", _I32), ("r", _I32), ("I", _P), ("rc", _I32)]


class InvJob(ctypes.Structure):
    _fields_ = [("T", _P), ("U", _P), ("n", _I32), ("r", _I32), ("I", _P), ("rc", _I32)]


class Block(ctypes.Structure):
    _fields_ = [("off", _U32), ("n", _U32), ("r", _U32), ("iout", _U32)]


class IBlock(ctypes.Structure):
    _fields_ = [("off", _U32), ("n", _U32), ("p0", _U32), ("pad", _U32)]


class Prof(ctypes.Structure):
    _fields_ = [("kernel", _I32), ("round", _I32), ("pass_", _I32), ("elems", _U32), ("segs", _U32),
                ("ms", ctypes.c_float)]


PLAIN = 1
OPT_SMALL_GROUP = 1
OPT_WARP_PATH = 2
OPT_LSD_ROUND0 = 3
OPT_LSD_BYTES = 4
OPT_CHAIN_FROM = 5
REQ_FWD = 1
REQ_INV = 2


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("cancelled", ctypes.c_int64), ("batches", ctypes.c_int64), ("bytes", ctypes.c_uint64),
                ("hbm_in_use", ctypes.c_uint64), ("hbm_peak", ctypes.c_uint64)]

_lib = None


def lib_path() -> str:
    """The library to load: $KGBWT_LIB when set (an explicit build, e.g. for side-by-side timing), else the
    bounds-checked build when KGBWT_CHECKED=1, else the release build."""
    if os.environ.get("KGBWT_LIB"):
        return os.environ["KGBWT_LIB"]
    return _build.LIB_CHECKED if os.environ.get("KGBWT_CHECKED") == "1" else _build.LIB


def lib():
    """The loaded C-ABI library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"kgbwt CUDA library not built: {path} (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    L.kolmo_sais_bwt_aux.argtypes = [_P, _P, _P, _I32, _I32, _P, _I32]
    L.kolmo_sais_bwt_aux.restype = _I32
    L.kolmo_sais_unbwt_aux.argtypes = [_P, _P, _P, _I32, _I32, _P, _I32]
    L.kolmo_sais_unbwt_aux.restype = _I32
    L.kolmo_sais_unbwt.argtypes = [_P, _P, _P, _I32, _I32, _I32]
    L.kolmo_sais_unbwt.restype = _I32
    L.kgbwt_fwd_batch.argtypes = [ctypes.POINTER(FwdJob), _I32, _U32]
    L.kgbwt_fwd_batch.restype = _I32
    L.kgbwt_inv_batch.argtypes = [ctypes.POINTER(InvJob), _I32, _U32]
    L.kgbwt_inv_batch.restype = _I32
    L.kgbwt_engine_create.restype = _P
    L.kgbwt_engine_destroy.argtypes = [_P]
    L.kgbwt_engine_config.argtypes = [_P, _I32, _I32, _I32]
    L.kgbwt_engine_config.restype = _I32
    L.kgbwt_engine_option.argtypes = [_P, _I32, _I32]
    L.kgbwt_engine_option.restype = _I32
    L.kgbwt_engine_fwd.argtypes = [_P, _P, _P, _P, _P, ctypes.POINTER(Block), _I32, _P, _U32]
    L.kgbwt_engine_fwd.restype = _I32
    L.kgbwt_engine_inv.argtypes = [_P, _P, _P, ctypes.POINTER(IBlock), _I32, _P, _U32]
    L.kgbwt_engine_inv.restype = _I32
    L.kgbwt_engine_wait.argtypes = [_P, _P]
    L.kgbwt_engine_wait.restype = _I32
    L.kgbwt_engine_stats.argtypes = [_P, _P, _P, _P]
    L.kgbwt_engine_stats.restype = _I32
    L.kgbwt_engine_workspace_bytes.argtypes = [_P]
    L.kgbwt_engine_workspace_bytes.restype = ctypes.c_uint64
    L.kgbwt_engine_profile.argtypes = [_P, _I32]
    L.kgbwt_engine_profile.restype = _I32
    L.kgbwt_engine_profile_read.argtypes = [_P, ctypes.POINTER(Prof), _I32]
    L.kgbwt_engine_profile_read.restype = _I32
    L.kgbwt_kernel_name.argtypes = [_I32]
    L.kgbwt_kernel_name.restype = ctypes.c_char_p
    L.kgbwt_dropin_stats.argtypes = [_P, _I32]
    L.kgbwt_dropin_stats.restype = _I32
    L.kgbwt_unbwt_noalloc.argtypes = [_P, _P, _I32, _I32, _P]
    L.kgbwt_unbwt_noalloc.restype = _I32
    L.kgbwt_server_create.argtypes = [_I32, ctypes.c_uint64, ctypes.c_uint64]
    L.kgbwt_server_create.restype = _P
    L.kgbwt_server_destroy.argtypes = [_P]
    L.kgbwt_server_submit.argtypes = [_P, _I32, _P, _P, _P, _I32, _I32]
    L.kgbwt_server_submit.restype = ctypes.c_int64
    L.kgbwt_server_wait.argtypes = [_P, ctypes.c_int64, _I32, _P, _P]
    L.kgbwt_server_wait.restype = _I32
    L.kgbwt_server_cancel.argtypes = [_P, ctypes.c_int64]
    L.kgbwt_server_cancel.restype = _I32
    L.kgbwt_server_stats_read.argtypes = [_P, ctypes.POINTER(ServerStats)]
    L.kgbwt_server_stats_read.restype = _I32
    L.kgbwt_server_inject_oom.argtypes = [_P, _I32]
    L.kgbwt_server_inject_oom.restype = _I32
    L.kgbwt_server_plan.argtypes = [_P, _P, _P, _I32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                    ctypes.c_uint64, _P]
    L.kgbwt_server_plan.restype = _I32
    L.kgbwt_estimate_bytes.argtypes = [_I32, _P, _P, _I32]
    L.kgbwt_estimate_bytes.restype = ctypes.c_uint64
    L.kgbwt_engine_last_config.argtypes = [_P, _P]
    L.kgbwt_engine_last_config.restype = _I32
    L.kgbwt_tuning_load.argtypes = [ctypes.c_char_p]
    L.kgbwt_tuning_load.restype = _I32
    L.kgbwt_tuning_lookup.argtypes = [ctypes.c_uint64, _P]
    L.kgbwt_tuning_lookup.restype = _I32
    L.kgbwt_tuning_lookup_n.argtypes = [ctypes.c_uint64, _P, _I32]
    L.kgbwt_tuning_lookup_n.restype = _I32
    L.kgbwt_engine_last_config_n.argtypes = [_P, _P, _I32]
    L.kgbwt_engine_last_config_n.restype = _I32
    L.libcubwt_allocate_device_storage.argtypes = [_P, ctypes.c_int64]
    L.libcubwt_allocate_device_storage.restype = ctypes.c_int64
    L.libcubwt_free_device_storage.argtypes = [_P]
    L.libcubwt_free_device_storage.restype = ctypes.c_int64
    L.libcubwt_bwt_aux.argtypes = [_P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P]
    L.libcubwt_bwt_aux.restype = ctypes.c_int64
    L.libcubwt_bwt.argtypes = [_P, _P, _P, ctypes.c_int64]
    L.libcubwt_bwt.restype = ctypes.c_int64
    L.libcubwt_unbwt.argtypes = [_P, _P, _P, ctypes.c_int64, _P, _I32]
    L.libcubwt_unbwt.restype = ctypes.c_int64
    L.kgbwt_last_error.restype = ctypes.c_char_p
    L.kgbwt_version.restype = _I32
    _lib = L
    return L


def last_error() -> str:
    return lib().kgbwt_last_error().decode(errors="replace")


# the exported symbols include/kgbwt.h declares (the CPU tests check that the library exports each of them)
EXPORTS = (
    "kolmo_sais_bwt_aux", "kolmo_sais_unbwt_aux", "kolmo_sais_unbwt", "kgbwt_fwd_batch", "kgbwt_inv_batch",
    "kgbwt_engine_create", "kgbwt_engine_destroy", "kgbwt_engine_config", "kgbwt_engine_fwd", "kgbwt_engine_inv",
    "kgbwt_engine_wait", "kgbwt_engine_stats", "kgbwt_engine_workspace_bytes", "kgbwt_last_error", "kgbwt_version",
    "kgbwt_engine_profile", "kgbwt_engine_profile_read", "kgbwt_kernel_name", "kgbwt_engine_option",
    "kgbwt_unbwt_noalloc", "kgbwt_dropin_stats", "kgbwt_server_create", "kgbwt_server_destroy", "kgbwt_server_submit", "kgbwt_server_wait",
    "kgbwt_server_cancel", "kgbwt_server_stats_read", "kgbwt_server_inject_oom", "kgbwt_server_plan",
    "kgbwt_estimate_bytes", "kgbwt_engine_last_config", "kgbwt_tuning_load", "kgbwt_tuning_lookup",
    "kgbwt_tuning_lookup_n", "kgbwt_engine_last_config_n",
    "libcubwt_allocate_device_storage", "libcubwt_free_device_storage", "libcubwt_bwt_aux", "libcubwt_bwt",
    "libcubwt_unbwt",
)
