"""Engine calls on device-resident buffers (torch CUDA tensors) and caller streams."""
import numpy as np
import pytest

import oracle as O
from kolmo_gb300 import codec
from kolmo_gb300 import workloads as W

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
