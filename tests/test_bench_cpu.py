"""The benchmark's roofline arithmetic without a GPU: the doubling model's algorithmic bytes per launch and the
per-round table that bench.py builds from a plain-path profile."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _rec(kernel, rnd, elems, ms):
    return {"kernel": kernel, "round": rnd, "pass": -1, "elems": elems, "segs": 0, "ms": ms}


def test_doubling_model_bytes_per_launch():
    n = 1 << 20
    # round 0: 33 B per suffix over all its radix passes, in equal parts
    assert bench.algorithmic_bytes(_rec("lsd_pass", 0, n, 1.0), 16, n) == pytest.approx(33.0 * n / 16)
    # rank rounds: 48 B per active suffix, credited to the kernel that sorts it
    for k in ("group_thread", "group_warp", "tile_sort_rank", "keygen"):
        assert bench.algorithmic_bytes(_rec(k, 2, 1000, 1.0), 16, n) == 48.0 * 1000
    # the inverse: 10 B per byte, half to the psi build and half to the walk
    assert bench.algorithmic_bytes(_rec("inv_walk", 0, n, 1.0), 16, n) == 5.0 * n
    assert bench.algorithmic_bytes(_rec("inv_scatter", 0, n, 1.0), 16, n) == 5.0 * n
    # overhead kernels get none
    for k in ("seg_count", "seg_rank", "fixup", "msd_scatter", "chain", "control"):
        assert bench.algorithmic_bytes(_rec(k, 1, n, 1.0), 16, n) == 0.0


def test_per_round_table():
    n = 1 << 24
    prof_f = [_rec("lsd_pass", 0, n, 0.5) for _ in range(16)] + [_rec("seg_count", 0, n, 2.0)]
    prof_f += [_rec("group_thread", 1, 3_000_000, 1.0), _rec("group_warp", 1, 1_000_000, 0.5),
               _rec("tile_sort_rank_keyed", 1, 500_000, 0.25), _rec("fixup", 1, n, 0.25)]
    prof_f += [_rec("group_thread", 2, 1_000_000, 0.5)]
    prof_i = [_rec("inv_scatter", 0, n, 0.4), _rec("inv_walk", 0, n, 1.6)]
    peak = 6800.0
    by_kernel, table = bench.profile_table(prof_f, prof_i, n, 16, peak)
    assert [r["round"] for r in table] == [0, 1, 2]
    r0, r1, r2 = table
    # round 0: every suffix, 33 B each, over the whole round's time (passes and segmentation)
    assert r0["m"] == n and r0["ms"] == pytest.approx(10.0)
    assert r0["GBs"] == pytest.approx(33.0 * n / 10e-3 / 1e9, rel=1e-3)
    assert r0["frac"] == pytest.approx(r0["GBs"] / peak, abs=1e-4)
    # round 1: the sort kernels' suffixes (the keyed tiles sort buckets of the large list and are not counted again)
    assert r1["m"] == 4_000_000 and r1["h"] == 16 and r1["ms"] == pytest.approx(2.0)
    assert r1["GBs"] == pytest.approx(48.0 * 4_000_000 / 2e-3 / 1e9, rel=1e-3)
    assert r2["h"] == 32 and r2["m"] == 1_000_000
    # per kernel: the radix pass holds round 0's 33 B per suffix, the inverse its 10 B per byte
    assert by_kernel["lsd_pass"]["launches"] == 16
    assert by_kernel["lsd_pass"]["bytes"] == pytest.approx(33.0 * n)
    assert by_kernel["inv_walk"]["bytes"] + by_kernel["inv_scatter"]["bytes"] == pytest.approx(10.0 * n)
    assert by_kernel["fixup"]["bytes"] == 0.0
