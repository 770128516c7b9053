"""Autotuner of the forward sort: times candidate configurations on this GPU for batches of several sizes and writes
the tuning table (JSON, one bucket per batch size) that the library loads (kgbwt_tuning_load, KGBWT_TUNING, or
tuning_gb300.json beside this package). Results never depend on the configuration; only the time does.

    python -m kolmo_gb300.autotune --out kolmo_gb300/tuning_gb300.json [--reps 3] [--quick]

Tuned per bucket: CTAs per SM of the block tile kernel (tile_ctas) and of the bucket passes (msd_ctas), the
counting-sort threshold of the tile kernel (small_group), the warp-level tile path (warp_path), the round-0 path
(lsd_round0: one LSD radix sort of all suffixes, or bucket passes + tiles), the prefix it sorts (lsd_bytes: 16,
which spares the first rank round, 12 or 8) and whether rank rounds follow repeat chains (chain_from: 1 or 0). The
tile capacity changes the workspace layout and is left at its default.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import sys

import numpy as np

from . import codec
from . import workloads as W
from .host import codec18_rlog, n_samples

MIB = 1 << 20

# (measured batch: list of (source, bytes)) per bucket; a bucket covers batches up to twice its measured size
BUCKETS = [
    ("prose 1 MiB", [("prose", 1 * MIB)]),
    ("prose 4 MiB", [("prose", 4 * MIB)]),
    ("prose 16 MiB", [("prose", 16 * MIB)]),
    ("prose 64 MiB", [("prose", 64 * MIB)]),
    ("96 mixed blocks, log-uniform 16 KiB-16 MiB", "mixed96"),
]

CANDIDATES = {
    "lsd_round0": (1, 0),
    "lsd_bytes": (16, 12, 8),
    "msd_ctas": (8, 4),
    "tile_ctas": (2, 1),
    "small_group": (64, 0),
    "warp_path": (1, 0),
    "chain_from": (1, 0),
}


def _batch(spec, seed):
    if spec == "mixed96":  # the mixed batch's shape (sources and size law) on another seed
        return [t for _, t in W.mixed_batch(96, seed=seed)]
    texts = []
    for k, (src, n) in enumerate(spec):
        texts.append(W.zipf_prose(n, seed + k) if src == "prose" else W.source_block(src, n, seed + k))
    return texts


def _time_config(texts, cfg, reps):
    """Median forward time (ms, graph path, CUDA events) of the batch under one configuration."""
    import torch

    offs, o = [], 0
    for t in texts:
        offs.append(o)
        o += (t.size + 15) // 16 * 16
    buf = np.zeros(o + 64, np.uint8)
    for t, off in zip(texts, offs):
        buf[off:off + t.size] = t
    blocks, k = [], 0
    for t, off in zip(texts, offs):
        r = 1 << codec18_rlog(int(t.size))
        blocks.append((off, int(t.size), r, k))
        k += n_samples(int(t.size), r)
    dT = torch.from_numpy(buf).cuda()
    dL = torch.zeros(o + len(texts) + 64, dtype=torch.uint8, device="cuda")
    dI = torch.zeros(k, dtype=torch.int32, device="cuda")
    eng = codec.Engine()
    eng.config(0, cfg["tile_ctas"], cfg["msd_ctas"], cfg["small_group"], cfg["warp_path"], cfg["lsd_round0"],
               cfg["lsd_bytes"], cfg["chain_from"])
    s = torch.cuda.Stream()
    times = []
    ref = None
    for it in range(reps + 2):  # call 0 runs plain (a new shape), call 1 captures the graph, the rest are timed
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        if eng.fwd(dT, dL, dI, blocks, stream=s) or eng.wait()[0]:
            raise RuntimeError("forward failed during tuning")
        e1.record(s)
        s.synchronize()
        if it >= 2:
            times.append(e0.elapsed_time(e1))
        if ref is None:
            ref = dI.cpu().numpy().copy()
    assert np.array_equal(ref, dI.cpu().numpy())  # same result under every configuration
    eng.close()
    return statistics.median(times), ref


def candidate_grid(quick: bool = False) -> list:
    """Every configuration the tuner times (the prefix width only varies on the LSD round 0); quick: the first four."""
    keys = list(CANDIDATES)
    grid = [dict(zip(keys, vals)) for vals in itertools.product(*(CANDIDATES[k] for k in keys))]
    grid = [g for g in grid if g["lsd_round0"] or g["lsd_bytes"] == CANDIDATES["lsd_bytes"][0]]
    return grid[:4] if quick else grid


def default_config() -> dict:
    """The library's defaults: each field's first candidate."""
    return {k: v[0] for k, v in CANDIDATES.items()}


def tune(reps: int = 3, quick: bool = False, log=print):
    import torch

    grid = candidate_grid(quick)
    default = default_config()
    buckets = []
    for bi, (name, spec) in enumerate(BUCKETS if not quick else BUCKETS[:2]):
        texts = _batch(spec, 0x5EED + 97 * bi)
        total = sum(int(t.size) for t in texts)
        results = []
        ref = None
        for cfg in grid:
            ms, out = _time_config(texts, cfg, reps)
            if ref is None:
                ref = out
            assert np.array_equal(ref, out), "configurations disagree"  # results never depend on the configuration
            results.append((ms, cfg))
        best_ms, best = min(results, key=lambda x: x[0])
        dflt_ms = next(ms for ms, c in results if c == default)
        log(f"{name}: best {best} {best_ms:.3f} ms (default {dflt_ms:.3f} ms)")
        buckets.append({"max_bytes": 2 * total, **best, "fwd_ms": round(best_ms, 4),
                        "default_fwd_ms": round(dflt_ms, 4), "workload": name})
    buckets[-1]["max_bytes"] = 1 << 40
    return {"version": 1, "device": torch.cuda.get_device_name(), "generated_by": "kolmo_gb300/autotune.py",
            "reps": reps, "buckets": buckets}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json"))
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--quick", action="store_true", help="two buckets, four candidates (a smoke run)")
    args = ap.parse_args(argv)
    # measure without any table: every candidate sets all tuned fields explicitly anyway
    codec.tuning_load(None)
    table = tune(args.reps, args.quick)
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print(f"wrote {args.out} ({len(table['buckets'])} buckets)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
