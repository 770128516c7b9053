"""Whole-frame parity of codec 18 (levels -8 and -9) with the GPU sorter linked into the reference's CLI.

Two binaries are built by ``oracle/Makefile`` (target ``frames``) from the reference's own sources, staged by
``oracle/stage_ref.py``: ``kolmo-ref``, the reference CLI with its sorter ``src/algo/sais/sais.c``, and ``kolmo-gpu``,
the same objects with ``libkgbwt.so`` linked in place of ``sais.c`` (the only callers, src/codecs/bwt_stream.c:52,
73-74, 233 and 294, are unchanged). Pinned three ways:

* the reference's determinism digests: the frames of the reference's seeded generator
  (benchmark/determinism/check.py) at -8 and -9, with 1 and 4 threads, must have the SHA-256 digests the reference
  pinned in benchmark/determinism/expected.sha256, and decode back;
* the reference CLI itself on seeded inputs of the benchmark's sources (the 1 MiB order-2 Markov block, Zipf word
  prose up to two 32 MiB blocks at -8, the -9 planner's slice trials): byte-identical frames, and each CLI decodes
  the other's frames;
* frames written by reference releases (tests/v12/*.kolmo) decode to the originals' digests (tests/v12.sha256).

``KGBWT_STATS`` makes the GPU library log its batches, which shows that the block sorts ran on the GPU."""
import hashlib
import os
import subprocess
import time

import numpy as np
import pytest

import stage_ref
from frame_inputs import determinism_inputs, expected_digests
from kolmo_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ORACLE = os.path.dirname(os.path.abspath(stage_ref.__file__))
TREE = stage_ref.staged() or stage_ref.stage()
if TREE is None:
    pytest.skip("the reference's sources are not staged (python oracle/stage_ref.py where the tree is mounted)",
                allow_module_level=True)


@pytest.fixture(scope="module")
def clis():
    r = subprocess.run(["make", "-C", ORACLE, f"REF={TREE}", "-j", str(os.cpu_count() or 4), "frames"],
                       capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    return os.path.join(ORACLE, "_ref", "kolmo-ref"), os.path.join(ORACLE, "_ref", "kolmo-gpu")


def _run(cmd, env=None):
    r = subprocess.run(cmd, capture_output=True, env=env)
    assert r.returncode == 0, (cmd, r.stderr.decode(errors="replace")[-500:])


def _sha(path: str) -> str:
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


class GpuLog:
    """KGBWT_STATS file of the GPU CLI: one line per batch the library ran."""

    def __init__(self, tmp):
        self.path = os.path.join(str(tmp), "kgbwt_stats.log")
        self.env = dict(os.environ, KGBWT_STATS=self.path)
        self.env.pop("KOLMO_MEMLIMIT", None)

    def lines(self):
        return open(self.path).read().splitlines() if os.path.exists(self.path) else []

    def calls(self, kind: str) -> int:
        return sum(int(x.split()[1].split("=")[1]) for x in self.lines() if x.startswith(kind))

    def sizes(self, kind: str) -> list:
        out = []
        for x in self.lines():
            if x.startswith(kind):
                field = [f for f in x.split() if f.startswith("sizes=")]
                out += [int(v) for v in field[0][6:].split(",") if v] if field else []
        return out


def test_determinism_digests_at_levels_8_and_9(clis, tmp_path):
    _, gpu = clis
    log = GpuLog(tmp_path)
    want = expected_digests(TREE)
    checked = 0
    inputs = determinism_inputs(TREE)
    for name, data in inputs:
        p = str(tmp_path / name)
        open(p, "wb").write(data)
        for level in ("-8", "-9"):
            digests = set()
            for t in ("1", "4"):
                z, back = p + ".k", p + ".back"
                _run([gpu, level, "-f", "-T", t, p, "-o", z], log.env)
                _run([gpu, "-d", "-f", z, "-o", back], log.env)
                assert open(back, "rb").read() == data, (name, level, t)
                digests.add(_sha(z))
            assert digests == {want[(name, level)]}, (name, level, digests)
            checked += 1
    assert checked == 2 * len(inputs) == 20  # ten seeded inputs, each at -8 and -9
    assert log.calls("fwd") > 0 and log.calls("inv") > 0, "no block was sorted by the GPU library"


def _int32_walk(n_values: int, seed: int) -> np.ndarray:
    """Binary data: a little-endian int32 random walk (the -9 planner codes a 512 KiB slice of each such block both
    ways before it decides, src/core/blocks.c:481-517)."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.integers(-50, 50, n_values)).astype("<i4").view(np.uint8)


def _frame_inputs():
    return [("markov1mib", W.markov2(1 << 20, 0xC0FFEE), ("-8", "-9"), ("1",), []),
            ("prose8mib", W.zipf_prose(8 << 20, 811), ("-8", "-9"), ("1", "4"), []),
            ("prose48mib", W.zipf_prose(48 << 20, 4811), ("-8",), ("4",), []),  # two blocks (32 + 16 MiB) at once
            ("acgt4mib", W.acgt(4 << 20, 77), ("-9",), ("1",), []),
            ("logs6mib", W.logs(6 << 20, 78), ("-8",), ("2",), []),
            ("int32walk96mib", _int32_walk(24 << 20, 6), ("-9",), ("8",), ["--block-size", "32"])]


def test_frames_equal_reference_cli(clis, tmp_path):
    ref, gpu = clis
    log = GpuLog(tmp_path)
    for name, T, levels, threads, extra in _frame_inputs():
        p = str(tmp_path / name)
        T.tofile(p)
        for level in levels:
            for t in threads:
                zr, zg = p + ".ref.k", p + ".gpu.k"
                _run([ref, level, "-f", "-T", t, *extra, p, "-o", zr])
                before = log.calls("fwd")
                _run([gpu, level, "-f", "-T", t, *extra, p, "-o", zg], log.env)
                assert log.calls("fwd") > before, (name, level, "no codec-18 block")
                assert open(zr, "rb").read() == open(zg, "rb").read(), (name, level, t)
                for dec, z in ((gpu, zr), (ref, zg), (gpu, zg)):
                    back = p + ".back"
                    _run([dec, "-d", "-f", z, "-o", back], log.env)
                    assert np.array_equal(np.fromfile(back, np.uint8), T), (name, level, t, dec)
    # the -9 planner's 512 KiB slice trials of the binary blocks went through the GPU sorter too
    assert (512 << 10) in log.sizes("fwd"), sorted(set(log.sizes("fwd")))


def test_corrupted_frames_fail_alike(clis, tmp_path):
    """On a string that is no BWT for its primary index the reference's decoders emit bytes that the block checksum
    rejects, where the GPU inverse returns -1, which the codec maps to KB_DATA_CORRUPT (src/codecs/bwt_stream.c:294).
    At the frame level the outcome must be the same: for single-byte corruptions throughout a -8 frame, both CLIs
    reject the same frames, and where both decode, they decode the same bytes."""
    ref, gpu = clis
    log = GpuLog(tmp_path)
    T = W.markov2(1 << 20, 0xBAD)
    p = str(tmp_path / "m1")
    T.tofile(p)
    z = p + ".k"
    _run([ref, "-8", "-f", p, "-o", z])
    frame = bytearray(open(z, "rb").read())
    rng = np.random.default_rng(31)
    positions = sorted(set(int(x) for x in rng.integers(0, len(frame), 24)) | set(range(16, 80, 4)))
    rejected = 0
    for pos in positions:
        bad = bytearray(frame)
        bad[pos] ^= 0x5A
        zb, outs = str(tmp_path / "bad.k"), {}
        open(zb, "wb").write(bytes(bad))
        for name, cli, env in (("reference", ref, None), ("gpu", gpu, log.env)):
            out = str(tmp_path / f"bad.{name}")
            if os.path.exists(out):
                os.remove(out)
            r = subprocess.run([cli, "-d", "-f", zb, "-o", out], capture_output=True, env=env)
            outs[name] = (r.returncode != 0, open(out, "rb").read() if r.returncode == 0 else None)
        assert outs["reference"][0] == outs["gpu"][0], (pos, outs["reference"][0], outs["gpu"][0])
        assert outs["reference"][1] == outs["gpu"][1], pos
        rejected += outs["reference"][0]
    assert rejected > 0
    print(f"\n{rejected} of {len(positions)} single-byte corruptions rejected by both CLIs")


def test_reference_release_frames_decode(clis, tmp_path):
    _, gpu = clis
    log = GpuLog(tmp_path)
    v12 = os.path.join(TREE, "tests", "v12")
    digests = {}
    for line in open(os.path.join(TREE, "tests", "v12.sha256")):
        parts = line.split()
        if len(parts) == 2:
            digests[parts[1]] = parts[0]
    decoded = 0
    for line in open(os.path.join(v12, "MANIFEST")):
        parts = line.split()
        if len(parts) != 2 or not os.path.exists(os.path.join(v12, parts[0])) or parts[1] not in digests:
            continue
        out = str(tmp_path / "out")
        _run([gpu, "-d", "-f", os.path.join(v12, parts[0]), "-o", out], log.env)
        assert _sha(out) == digests[parts[1]], parts[0]
        decoded += 1
    assert decoded >= 50
    assert log.calls("inv") > 0, "no frame of the corpus reached the GPU inverse"


def test_whole_frame_throughput(clis, tmp_path):
    """Whole -8 frames of a 256 MiB prose file (eight 32 MiB blocks, every host thread): the GPU CLI's frame equals
    the reference CLI's, and both decode it back. Prints the two CLIs' compress and decompress throughput (MiB/s of
    input, process start and the GPU's context creation included): LZP, QLFC and the container stay on the host
    cores in both, so this is the whole codec's speed, not the sorter's."""
    ref, gpu = clis
    log = GpuLog(tmp_path)
    T = W.zipf_prose(256 << 20, 2561)
    p = str(tmp_path / "prose256")
    T.tofile(p)
    t = str(os.cpu_count() or 1)
    res = {}
    for name, cli, env in (("reference", ref, None), ("gpu", gpu, log.env)):
        z, back = p + f".{name}.k", p + f".{name}.back"
        t0 = time.perf_counter()
        _run([cli, "-8", "-f", "-T", t, p, "-o", z], env)
        t1 = time.perf_counter()
        _run([cli, "-d", "-f", "-T", t, z, "-o", back], env)
        t2 = time.perf_counter()
        assert np.array_equal(np.fromfile(back, np.uint8), T), name
        res[name] = (T.size / 2**20 / (t1 - t0), T.size / 2**20 / (t2 - t1))
    assert open(p + ".reference.k", "rb").read() == open(p + ".gpu.k", "rb").read()
    assert log.calls("fwd") >= 8 and log.calls("inv") >= 8
    batches = [x for x in log.lines() if x.startswith("fwd")]
    print(f"\nwhole -8 frames, 256 MiB prose, -T {t}: reference CLI compress {res['reference'][0]:.1f} MiB/s, "
          f"decompress {res['reference'][1]:.1f} MiB/s; GPU CLI compress {res['gpu'][0]:.1f} MiB/s, decompress "
          f"{res['gpu'][1]:.1f} MiB/s; {log.calls('fwd')} forward calls in {len(batches)} batches")
