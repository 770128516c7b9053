"""Host-side mirror of the reference's suffix-sorter interface for the BWT path (adnaneben/kolmo
src/algo/sais/sais.h:10-20), on the GPU engine.

``bwt_aux`` / ``unbwt_aux`` / ``unbwt`` keep the reference's argument meaning and return codes (0, -1 bad arguments
or indexes out of range, -2 out of memory); they return the output arrays alongside the code. ``fwd_batch`` and
``inv_batch`` run many blocks in one device pass. ``Engine`` works on device-resident buffers (torch tensors) on a
caller stream. Every call goes through the C ABI of ``libkgbwt.so``; nothing here computes a BWT on the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native

_DUMMY_A = np.zeros(1, np.int32)  # the caller's scratch: checked for NULL like the reference, never touched


def n_samples(n: int, r: int) -> int:
    return (n - 1) // r + 1 if n > 0 and r > 0 else 1


def _u8(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint8)
    return a if a.size else np.zeros(1, np.uint8)


def bwt_aux(T, r: int):
    """kolmo_sais_bwt_aux: returns (rc, U, I)."""
    T = np.ascontiguousarray(T, dtype=np.uint8)
    n = int(T.size)
    Tb = _u8(T)
    U = np.zeros(max(n, 1), np.uint8)
    I = np.zeros(max(n_samples(n, r), 1), np.int32)
    rc = native.lib().kolmo_sais_bwt_aux(Tb.ctypes.data, U.ctypes.data, _DUMMY_A.ctypes.data, n, r, I.ctypes.data, 1)
    return int(rc), U[:n], I[: n_samples(n, r)]


def unbwt_aux(U, r: int, I):
    """kolmo_sais_unbwt_aux: returns (rc, T)."""
    U = np.ascontiguousarray(U, dtype=np.uint8)
    n = int(U.size)
    Ub = _u8(U)
    I = np.ascontiguousarray(I, dtype=np.int32)
    out = np.zeros(max(n, 1), np.uint8)
    rc = native.lib().kolmo_sais_unbwt_aux(Ub.ctypes.data, out.ctypes.data, _DUMMY_A.ctypes.data, n, r,
                                           I.ctypes.data, 1)
    return int(rc), out[:n]


def unbwt(U, idx: int):
    """kolmo_sais_unbwt: returns (rc, T)."""
    U = np.ascontiguousarray(U, dtype=np.uint8)
    n = int(U.size)
    Ub = _u8(U)
    out = np.zeros(max(n, 1), np.uint8)
    rc = native.lib().kolmo_sais_unbwt(Ub.ctypes.data, out.ctypes.data, _DUMMY_A.ctypes.data, n, idx, 1)
    return int(rc), out[:n]


def dropin_stats() -> dict:
    """Coalescing counters of the drop-in and batch calls (kgbwt_dropin_stats)."""
    out = (ctypes.c_int64 * 7)()
    native.lib().kgbwt_dropin_stats(ctypes.addressof(out), 7)
    keys = ("fwd_calls", "fwd_batches", "fwd_largest", "inv_calls", "inv_batches", "inv_largest", "retried")
    return dict(zip(keys, (int(x) for x in out)))


def fwd_batch(blocks, plain: bool = False):
    """blocks: list of (T, r). Returns (rc, [(rc_i, U_i, I_i)])."""
    keep, jobs = [], (native.FwdJob * max(len(blocks), 1))()
    outs = []
    for k, (T, r) in enumerate(blocks):
        T = _u8(T) if np.asarray(T).size else np.zeros(1, np.uint8)
        n = int(np.asarray(blocks[k][0]).size)
        U = np.zeros(max(n, 1), np.uint8)
        I = np.zeros(max(n_samples(n, r), 1), np.int32)
        keep += [T, U, I]
        jobs[k].T, jobs[k].U, jobs[k].n, jobs[k].r, jobs[k].I = T.ctypes.data, U.ctypes.data, n, r, I.ctypes.data
        outs.append((U, I, n, r))
    rc = native.lib().kgbwt_fwd_batch(jobs, len(blocks), native.PLAIN if plain else 0)
    res = [(int(jobs[k].rc), U[:n], I[: n_samples(n, r)]) for k, (U, I, n, r) in enumerate(outs)]
    return int(rc), res


def inv_batch(blocks, plain: bool = False):
    """blocks: list of (U, r, I). Returns (rc, [(rc_i, T_i)])."""
    keep, jobs = [], (native.InvJob * max(len(blocks), 1))()
    outs = []
    for k, (U, r, I) in enumerate(blocks):
        n = int(np.asarray(U).size)
        Ub = _u8(U)
        Ib = np.ascontiguousarray(I, dtype=np.int32)
        out = np.zeros(max(n, 1), np.uint8)
        keep += [Ub, Ib, out]
        jobs[k].T, jobs[k].U, jobs[k].n, jobs[k].r, jobs[k].I = Ub.ctypes.data, out.ctypes.data, n, r, Ib.ctypes.data
        outs.append((out, n))
    rc = native.lib().kgbwt_inv_batch(jobs, len(blocks), native.PLAIN if plain else 0)
    return int(rc), [(int(jobs[k].rc), out[:n]) for k, (out, n) in enumerate(outs)]


class Engine:
    """A device engine (one batch in flight). Buffers are torch CUDA tensors; calls enqueue on `stream`
    (a torch.cuda.Stream or None for the current stream) and `wait()` synchronises and reports errors."""

    def __init__(self, tile_cap: int = 0, tile_ctas: int = 0, msd_ctas: int = 0):
        self.h = native.lib().kgbwt_engine_create()
        if not self.h:
            raise MemoryError("kgbwt_engine_create failed")
        if tile_cap or tile_ctas or msd_ctas:
            self.config(tile_cap, tile_ctas, msd_ctas)

    def config(self, tile_cap: int = 0, tile_ctas: int = 0, msd_ctas: int = 0, small_group: int = -1,
               warp_path: int = -1, lsd_round0: int = -1, lsd_bytes: int = -1, chain_from: int = -1):
        L = native.lib()
        rc = L.kgbwt_engine_config(self.h, tile_cap, tile_ctas, msd_ctas)
        for opt, val in ((native.OPT_SMALL_GROUP, small_group), (native.OPT_WARP_PATH, warp_path),
                         (native.OPT_LSD_ROUND0, lsd_round0), (native.OPT_LSD_BYTES, lsd_bytes),
                         (native.OPT_CHAIN_FROM, chain_from)):
            if rc == 0 and val >= 0:
                rc = L.kgbwt_engine_option(self.h, opt, val)
        if rc:
            raise ValueError(f"bad engine config {tile_cap} {tile_ctas} {msd_ctas} {small_group} {warp_path} "
                             f"{lsd_round0} {lsd_bytes}")

    def close(self):
        if self.h:
            native.lib().kgbwt_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _stream(stream):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        return ctypes.c_void_p(s.cuda_stream)

    def fwd(self, dT, dL, dI, blocks, dSA=None, stream=None, plain: bool = False) -> int:
        """blocks: sequence of (off, n, r, iout)."""
        arr = (native.Block * len(blocks))(*[native.Block(*b) for b in blocks])
        return int(native.lib().kgbwt_engine_fwd(self.h, dT.data_ptr(), dL.data_ptr(), dI.data_ptr(),
                                                 dSA.data_ptr() if dSA is not None else None, arr, len(blocks),
                                                 self._stream(stream), native.PLAIN if plain else 0))

    def inv(self, dU, dOut, blocks, stream=None, plain: bool = False) -> int:
        """blocks: sequence of (off, n, p0)."""
        arr = (native.IBlock * len(blocks))(*[native.IBlock(b[0], b[1], b[2], 0) for b in blocks])
        return int(native.lib().kgbwt_engine_inv(self.h, dU.data_ptr(), dOut.data_ptr(), arr, len(blocks),
                                                 self._stream(stream), native.PLAIN if plain else 0))

    def wait(self, nblocks: int = 0):
        st = np.zeros(max(nblocks, 1), np.int32)
        rc = native.lib().kgbwt_engine_wait(self.h, st.ctypes.data)
        return int(rc), st[:nblocks]

    def stats(self):
        r, p, l = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        native.lib().kgbwt_engine_stats(self.h, ctypes.byref(r), ctypes.byref(p), ctypes.byref(l))
        return {"rounds": r.value, "passes": p.value, "launches": l.value}

    def profile(self, enable: bool = True):
        native.lib().kgbwt_engine_profile(self.h, 1 if enable else 0)

    def profile_read(self):
        """Records of the last plain-path call: list of dicts (kernel, round, pass, elems, segs, ms)."""
        L = native.lib()
        n = L.kgbwt_engine_profile_read(self.h, None, 0)
        buf = (native.Prof * max(n, 1))()
        n = L.kgbwt_engine_profile_read(self.h, buf, n)
        return [{"kernel": L.kgbwt_kernel_name(r.kernel).decode(), "round": r.round, "pass": r.pass_,
                 "elems": r.elems, "segs": r.segs, "ms": r.ms} for r in buf[:n]]

    def last_config(self) -> dict:
        """The configuration the last forward call ran with (caller settings over the tuning table)."""
        c = np.zeros(len(CONFIG_FIELDS), np.int32)
        native.lib().kgbwt_engine_last_config_n(self.h, c.ctypes.data, len(CONFIG_FIELDS))
        return dict(zip(CONFIG_FIELDS, (int(x) for x in c)))

    def workspace_bytes(self) -> int:
        return int(native.lib().kgbwt_engine_workspace_bytes(self.h))


CONFIG_FIELDS = ("tile_cap", "tile_ctas", "msd_ctas", "small_group", "warp_path", "lsd_round0", "lsd_bytes",
                 "chain_from")


def tuning_load(path) -> int:
    """Replaces the tuning table (None: no table); returns the number of buckets or -1."""
    return int(native.lib().kgbwt_tuning_load(None if path is None else str(path).encode()))


def tuning_lookup(n: int):
    """(from_table, config) that a batch of n bytes would run with."""
    c = np.zeros(len(CONFIG_FIELDS), np.int32)
    t = int(native.lib().kgbwt_tuning_lookup_n(n, c.ctypes.data, len(CONFIG_FIELDS)))
    return t == 1, dict(zip(CONFIG_FIELDS, (int(x) for x in c)))


class Server:
    """The request server (kgbwt_server_*): forward and inverse BWT requests on host arrays, batched as they arrive
    onto `slots` workers with their own streams, admitted against an HBM budget (0: none)."""

    def __init__(self, slots: int = 2, hbm_budget: int = 0, max_batch_bytes: int = 0):
        self.h = native.lib().kgbwt_server_create(slots, hbm_budget, max_batch_bytes)
        if not self.h:
            raise RuntimeError("kgbwt_server_create failed")
        self._keep = {}

    def submit_fwd(self, T, r: int):
        """Queues the forward BWT of T with sampling interval r; returns (id, U, I) (filled on completion)."""
        T = _u8(T)
        n = int(T.size)
        U = np.zeros(max(n, 1), np.uint8)
        I = np.zeros(max(n_samples(n, r), 1), np.int32)
        rid = int(native.lib().kgbwt_server_submit(self.h, native.REQ_FWD, T.ctypes.data, U.ctypes.data,
                                                   I.ctypes.data, n, r))
        if rid < 0:
            raise ValueError("bad forward request")
        self._keep[rid] = (T, U, I)
        return rid, U[:n], I[: n_samples(n, r)]

    def submit_inv(self, U, r: int, I):
        """Queues the inverse BWT of U (sampled indexes I, interval r); returns (id, T) (filled on completion)."""
        U = _u8(U)
        n = int(U.size)
        Ib = np.ascontiguousarray(I, dtype=np.int32)
        out = np.zeros(max(n, 1), np.uint8)
        rid = int(native.lib().kgbwt_server_submit(self.h, native.REQ_INV, U.ctypes.data, out.ctypes.data,
                                                   Ib.ctypes.data, n, r))
        if rid < 0:
            raise ValueError("bad inverse request")
        self._keep[rid] = (U, Ib, out)
        return rid, out[:n]

    def wait(self, rid: int, timeout_ms: int = -1):
        """Returns (status, rc, latency_us): status 1 done, 0 timeout, -1 unknown id."""
        rc, lat = ctypes.c_int32(0), ctypes.c_double(0.0)
        st = int(native.lib().kgbwt_server_wait(self.h, rid, timeout_ms, ctypes.byref(rc), ctypes.byref(lat)))
        if st == 1:
            self._keep.pop(rid, None)
        return st, int(rc.value), float(lat.value)

    def cancel(self, rid: int) -> int:
        return int(native.lib().kgbwt_server_cancel(self.h, rid))

    def inject_oom(self, batches: int) -> int:
        return int(native.lib().kgbwt_server_inject_oom(self.h, batches))

    def stats(self) -> dict:
        s = native.ServerStats()
        native.lib().kgbwt_server_stats_read(self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in native.ServerStats._fields_}

    def close(self):
        if self.h:
            native.lib().kgbwt_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def server_plan(kinds, sizes, rs, have_fwd: int, have_inv: int, avail: int, max_batch_bytes: int = 0):
    """The server's batching policy on its own: indexes of the pending requests it would batch next."""
    k = np.ascontiguousarray(kinds, np.int32)
    n = np.ascontiguousarray(sizes, np.int32)
    r = np.ascontiguousarray(rs, np.int32)
    take = np.zeros(max(len(k), 1), np.int32)
    c = native.lib().kgbwt_server_plan(k.ctypes.data, n.ctypes.data, r.ctypes.data, len(k), have_fwd, have_inv,
                                       avail, max_batch_bytes, take.ctypes.data)
    return list(take[:c]) if c >= 0 else None


def estimate_bytes(kind: int, sizes, rs) -> int:
    """Device bytes a fresh worker needs for one batch of these requests."""
    n = np.ascontiguousarray(sizes, np.int32)
    r = np.ascontiguousarray(rs, np.int32)
    return int(native.lib().kgbwt_estimate_bytes(kind, n.ctypes.data, r.ctypes.data, len(n)))
