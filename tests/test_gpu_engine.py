"""Engine calls on device-resident buffers (torch CUDA tensors) and caller streams."""
import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec
from kolmo_gb300 import workloads as W
import refgen as R

pytestmark = pytest.mark.gpu


def _pack(texts):
    offs, o = [], 0
    for t in texts:
        offs.append(o)
        o += (t.size + 15) // 16 * 16
    buf = np.zeros(o + 64, np.uint8)
    for t, off in zip(texts, offs):
        buf[off:off + t.size] = t
    return buf, offs


def test_engine_forward_inverse_on_stream():
    import torch

    texts = [W.source_block(i % 3, 50_000 + 40_000 * i, i) for i in range(6)]
    buf, offs = _pack(texts)
    r = 1 << 12
    iouts, k = [], 0
    for t in texts:
        iouts.append(k)
        k += (t.size - 1) // r + 1
    dT = torch.from_numpy(buf).cuda()
    dL = torch.zeros(buf.size + len(texts), dtype=torch.uint8, device="cuda")
    dI = torch.zeros(k, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    eng = codec.Engine()
    blocks = [(off, t.size, r, io) for t, off, io in zip(texts, offs, iouts)]
    assert eng.fwd(dT, dL, dI, blocks, stream=s) == 0
    assert eng.wait()[0] == 0
    st = eng.stats()
    assert st["rounds"] >= 1
    L = dL.cpu().numpy()
    I = dI.cpu().numpy()
    Us = []
    for b, (t, off, io) in enumerate(zip(texts, offs, iouts)):
        oU, oI = O.bwt_aux(t, r)[1:]
        ns = oI.size
        assert np.array_equal(I[io:io + ns], oI)
        col = L[off + b: off + b + t.size + 1]
        p0 = int(oI[0])
        U = np.concatenate([col[:p0], col[p0 + 1:]])
        assert np.array_equal(U, oU)
        Us.append(U)
    # inverse on device: BWT strings at the same offsets
    ubuf = np.zeros_like(buf)
    for U, off in zip(Us, offs):
        ubuf[off:off + U.size] = U
    dU = torch.from_numpy(ubuf).cuda()
    dOut = torch.zeros_like(dU)
    iblocks = [(off, t.size, int(I[io])) for t, off, io in zip(texts, offs, iouts)]
    assert eng.inv(dU, dOut, iblocks, stream=s) == 0
    rc, status = eng.wait(len(iblocks))
    assert rc == 0 and not status.any()
    out = dOut.cpu().numpy()
    for t, off in zip(texts, offs):
        assert np.array_equal(out[off:off + t.size], t)
    assert eng.workspace_bytes() > 0


def test_engine_configs_give_identical_results():
    import torch

    t = W.zipf_prose(3 << 20, 4)
    n = t.size
    dT = torch.zeros(n + 64, dtype=torch.uint8, device="cuda")
    dT[:n] = torch.from_numpy(t).cuda()
    ref = None
    for cap, tc, mc in ((4096, 2, 4), (8192, 1, 2), (4096, 1, 8)):
        eng = codec.Engine(cap, tc, mc)
        dL = torch.zeros(n + 1, dtype=torch.uint8, device="cuda")
        dI = torch.zeros(64, dtype=torch.int32, device="cuda")
        assert eng.fwd(dT, dL, dI, [(0, n, 1 << 19, 0)]) == 0 and eng.wait()[0] == 0
        got = (dL.cpu().numpy(), dI.cpu().numpy())
        if ref is None:
            ref = got
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


@pytest.mark.parametrize("lsd_round0,lsd_bytes", [(0, 16), (1, 8), (1, 12), (1, 16)])
def test_round0_paths_on_mixed_batch(lsd_round0, lsd_bytes):
    """Round 0 as one LSD radix sort of the batch (over 8-, 12- or 16-byte prefixes, sort tiles aligned to the blocks), or
    as bucket passes + tiles: each must give the oracle's L column and sampled indexes, on a batch that mixes two-byte
    blocks (the engine's minimum), blocks shorter than the prefix, runs longer than a tile (large groups spanning
    segmentation tiles) and ordinary text."""
    import torch

    texts = [np.array([7, 1], np.uint8), np.array([3, 3], np.uint8), np.full(20_000, 97, np.uint8),
             W.periodic(60_000, 11, 7, 1 << 14), W.markov2(90_000, 12), R.test_block(5, 5_000),
             np.array([5, 0, 5, 0, 5, 0, 5, 0, 5, 0, 5], np.uint8), np.zeros(3_000, np.uint8),
             W.zipf_prose(150_000, 13), np.array([2, 1, 2], np.uint8)]
    buf, offs = _pack(texts)
    r = 1 << 10
    iouts, k = [], 0
    for t in texts:
        iouts.append(k)
        k += (t.size - 1) // r + 1
    dT = torch.from_numpy(buf).cuda()
    dL = torch.zeros(buf.size + len(texts), dtype=torch.uint8, device="cuda")
    dI = torch.zeros(k, dtype=torch.int32, device="cuda")
    eng = codec.Engine()
    eng.config(lsd_round0=lsd_round0, lsd_bytes=lsd_bytes)
    blocks = [(off, t.size, r, io) for t, off, io in zip(texts, offs, iouts)]
    for it in range(3):  # plain launches (first sight of the shape), then capture, then the cached graph
        dL.zero_()
        assert eng.fwd(dT, dL, dI, blocks) == 0
        assert eng.wait()[0] == 0
        assert (eng.stats()["launches"] > 0) == (it == 0), it
        L = dL.cpu().numpy()
        I = dI.cpu().numpy()
        for b, (t, off, io) in enumerate(zip(texts, offs, iouts)):
            oU, oI = O.bwt_aux(t, r)[1:]
            assert np.array_equal(I[io:io + oI.size], oI), b
            col = L[off + b: off + b + t.size + 1]
            p0 = int(oI[0])
            assert np.array_equal(np.concatenate([col[:p0], col[p0 + 1:]]), oU), b


def _repeats(n, seed):
    """A random block with long verbatim repeats: stretches of 1-40 KiB copied from earlier positions, some copies of
    copies, some overlapping their source (periodic runs)."""
    rng = np.random.default_rng(seed)
    t = rng.integers(0, 4 if seed % 2 else 256, n).astype(np.uint8)
    for _ in range(40):
        L = int(rng.integers(1 << 10, 40 << 10))
        d = int(rng.integers(1, n - L))
        s = int(rng.integers(max(0, d - 3 * L), d))
        for q in range(0, L, max(1, d - s)):  # overlapping copies are made in steps of the distance
            m = min(d - s, L - q)
            t[d + q:d + q + m] = t[s + q:s + q + m]
    return t


@pytest.mark.parametrize("chain_from", [0, 1, 3])
def test_repeat_chains_give_the_doubling_order(chain_from):
    """Pairs ordered along their repeat chains (from rank round 1, from round 3, or never) give the oracle's BWT and
    sampled indexes on blocks made of long verbatim repeats, on the plain path and in the captured graph."""
    import torch

    texts = [_repeats(3 << 20, 1), _repeats(2 << 20, 2), W.zipf_prose(4 << 20, 71),
             np.concatenate([W.markov2(1 << 20, 5)] * 2), W.periodic(1 << 20, 9, 4096, 1 << 16)]
    buf, offs = _pack(texts)
    r = 1 << 14
    iouts, k = [], 0
    for t in texts:
        iouts.append(k)
        k += (t.size - 1) // r + 1
    want = [O.bwt_aux(t, r)[1:] for t in texts]
    dT = torch.from_numpy(buf).cuda()
    dL = torch.zeros(buf.size + len(texts), dtype=torch.uint8, device="cuda")
    dI = torch.zeros(k, dtype=torch.int32, device="cuda")
    eng = codec.Engine()
    eng.config(chain_from=chain_from)
    blocks = [(off, t.size, r, io) for t, off, io in zip(texts, offs, iouts)]
    for it in range(3):  # plain launches, then capture, then the cached graph
        dL.zero_()
        assert eng.fwd(dT, dL, dI, blocks) == 0
        assert eng.wait()[0] == 0
        L = dL.cpu().numpy()
        I = dI.cpu().numpy()
        for b, (t, off, io) in enumerate(zip(texts, offs, iouts)):
            oU, oI = want[b]
            assert np.array_equal(I[io:io + oI.size], oI), (chain_from, it, b)
            col = L[off + b: off + b + t.size + 1]
            p0 = int(oI[0])
            assert np.array_equal(np.concatenate([col[:p0], col[p0 + 1:]]), oU), (chain_from, it, b)


def test_tuning_table_applies_and_explicit_settings_win(tmp_path):
    import json
    import os

    import torch

    t = W.zipf_prose(2 << 20, 21)
    n = t.size
    dT = torch.zeros(n + 64, dtype=torch.uint8, device="cuda")
    dT[:n] = torch.from_numpy(t).cuda()
    table = {"buckets": [{"max_bytes": 1 << 40, "tile_ctas": 1, "msd_ctas": 3, "small_group": 0, "warp_path": 0,
                          "lsd_round0": 0, "lsd_bytes": 8}]}
    p = tmp_path / "tune.json"
    p.write_text(json.dumps(table))
    pkg = os.path.join(os.path.dirname(codec.__file__), "tuning_gb300.json")
    try:
        assert codec.tuning_load(p) == 1
        outs = []
        for explicit in (False, True):
            eng = codec.Engine()
            if explicit:
                eng.config(0, 2, 8, 64, 1, 1, 16)
            dL = torch.zeros(n + 1, dtype=torch.uint8, device="cuda")
            dI = torch.zeros(4, dtype=torch.int32, device="cuda")
            assert eng.fwd(dT, dL, dI, [(0, n, 1 << 20, 0)]) == 0 and eng.wait()[0] == 0
            c = eng.last_config()
            want = (2, 8, 64, 1, 1, 16) if explicit else (1, 3, 0, 0, 0, 8)
            assert (c["tile_ctas"], c["msd_ctas"], c["small_group"], c["warp_path"], c["lsd_round0"],
                    c["lsd_bytes"]) == want
            outs.append((dL.cpu().numpy(), dI.cpu().numpy()))
            eng.close()
        assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    finally:
        codec.tuning_load(pkg if os.path.exists(pkg) else None)
