"""The tuning table without a GPU: the library parses the autotuner's JSON, picks the bucket of a batch size, rejects
malformed tables, and reports the defaults when no table is loaded."""
import json
import os

import pytest

from kolmo_gb300 import codec

PKG_TABLE = os.path.join(os.path.dirname(codec.__file__), "tuning_gb300.json")


@pytest.fixture
def restore_table():
    yield
    codec.tuning_load(PKG_TABLE if os.path.exists(PKG_TABLE) else None)


def test_bucket_lookup(tmp_path, restore_table):
    t = {"version": 1, "device": "test", "buckets": [
        {"max_bytes": 1 << 30, "tile_ctas": 2, "msd_ctas": 4, "small_group": 0, "warp_path": 1, "lsd_round0": 0,
         "workload": "large"},
        {"max_bytes": 1 << 20, "tile_ctas": 1, "msd_ctas": 8, "small_group": 64, "warp_path": 0, "lsd_round0": 1,
         "fwd_ms": 0.5},
    ]}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(t))
    assert codec.tuning_load(p) == 2
    hit, c = codec.tuning_lookup(1000)
    assert hit and c["tile_ctas"] == 1 and c["msd_ctas"] == 8 and c["warp_path"] == 0 and c["lsd_round0"] == 1
    hit, c = codec.tuning_lookup(5 << 20)
    assert hit and c["tile_ctas"] == 2 and c["msd_ctas"] == 4 and c["small_group"] == 0 and c["lsd_round0"] == 0
    hit, c = codec.tuning_lookup(1 << 33)  # past every bucket: the last one
    assert hit and c["msd_ctas"] == 4
    assert c["tile_cap"] == 4096  # never tuned


def test_malformed_tables_are_refused(tmp_path, restore_table):
    for bad in ('{"no": []}', '{"buckets": [{"tile_ctas": 2}]}', '{"buckets": [{"max_bytes": 10, "msd_ctas": 99}]}',
                '{"buckets": [{"max_bytes": 10, "warp_path": 2}]}', '{"buckets": [{"max_bytes": 10, "lsd_bytes": 10}]}',
                'not json'):
        p = tmp_path / "bad.json"
        p.write_text(bad)
        assert codec.tuning_load(p) == -1
    assert codec.tuning_load(tmp_path / "missing.json") == -1


def test_prefix_widths(tmp_path, restore_table):
    """Round 0 sorts 8-, 12- or 16-byte prefixes; a bucket without the field keeps the default (16)."""
    t = {"buckets": [{"max_bytes": 1 << 20, "lsd_bytes": 12}, {"max_bytes": 1 << 22, "lsd_bytes": 8},
                     {"max_bytes": 1 << 30}]}
    p = tmp_path / "w.json"
    p.write_text(json.dumps(t))
    assert codec.tuning_load(p) == 3
    assert [codec.tuning_lookup(n)[1]["lsd_bytes"] for n in (1000, 2 << 20, 8 << 20)] == [12, 8, 16]


def test_no_table_gives_defaults(restore_table):
    assert codec.tuning_load(None) == 0
    hit, c = codec.tuning_lookup(64 << 20)
    assert not hit and c == {"tile_cap": 4096, "tile_ctas": 2, "msd_ctas": 8, "small_group": 64, "warp_path": 1,
                             "lsd_round0": 1, "lsd_bytes": 16, "chain_from": 1}


def test_chain_rounds_by_bucket(tmp_path, restore_table):
    """The first repeat-chain round is a per-bucket field (0: none; a bucket without it keeps the default, 1); values
    above 64 are refused."""
    t = {"buckets": [{"max_bytes": 1 << 20, "chain_from": 0}, {"max_bytes": 1 << 22, "chain_from": 3},
                     {"max_bytes": 1 << 30}]}
    p = tmp_path / "c.json"
    p.write_text(json.dumps(t))
    assert codec.tuning_load(p) == 3
    assert [codec.tuning_lookup(n)[1]["chain_from"] for n in (1000, 2 << 20, 8 << 20)] == [0, 3, 1]
    p.write_text(json.dumps({"buckets": [{"max_bytes": 10, "chain_from": 99}]}))
    assert codec.tuning_load(p) == -1


def test_config_report_lengths(restore_table):
    """The short report fills exactly its seven fields; the full one any prefix of the eight."""
    import numpy as np

    from kolmo_gb300 import native

    codec.tuning_load(None)
    c = np.full(9, -7, np.int32)
    assert native.lib().kgbwt_tuning_lookup(1000, c.ctypes.data) == 0
    assert list(c[7:]) == [-7, -7]
    c = np.full(9, -7, np.int32)
    assert native.lib().kgbwt_tuning_lookup_n(1000, c.ctypes.data, 3) == 0
    assert list(c[:3]) == [4096, 2, 8] and list(c[3:]) == [-7] * 6
    c = np.full(9, -7, np.int32)
    assert native.lib().kgbwt_tuning_lookup_n(1000, c.ctypes.data, 9) == 0
    assert c[7] == 1 and c[8] == -7
    assert native.lib().kgbwt_tuning_lookup_n(1000, c.ctypes.data, 0) == -1


def test_packaged_table_parses_if_present(restore_table):
    if not os.path.exists(PKG_TABLE):
        pytest.skip("no packaged table")
    with open(PKG_TABLE) as f:
        n = len(json.load(f)["buckets"])
    assert codec.tuning_load(PKG_TABLE) == n


def test_autotune_grid(restore_table):
    """The autotuner's candidate grid: every field the library's table accepts, the prefix width varied only on the
    LSD round 0, and the defaults (each field's first candidate) among the candidates."""
    from kolmo_gb300 import autotune

    assert set(autotune.CANDIDATES) == set(codec.CONFIG_FIELDS) - {"tile_cap"}
    grid = autotune.candidate_grid()
    default = autotune.default_config()
    assert default in grid
    # the defaults the tuner assumes are the library's own (no table loaded)
    codec.tuning_load(None)
    lib_default = codec.tuning_lookup(1 << 20)[1]
    assert all(lib_default[k] == v for k, v in default.items())
    assert all(g["lsd_bytes"] == 16 for g in grid if not g["lsd_round0"])
    assert len(grid) == len({tuple(sorted(g.items())) for g in grid})
