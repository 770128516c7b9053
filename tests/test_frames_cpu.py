"""The frame oracle on the CPU: the reference CLI that oracle/Makefile compiles from the reference's staged sources
(its own files, this repository's build rules) must write, at -8 and -9 with 1 and 4 threads, the frames whose
SHA-256 digests the reference pinned in benchmark/determinism/expected.sha256, and decode them back. The GPU frame
tests compare the GPU-linked CLI with exactly this binary, so this pins the comparison's reference side."""
import hashlib
import os
import subprocess

import pytest

import stage_ref
from frame_inputs import determinism_inputs, expected_digests

TREE = stage_ref.staged() or stage_ref.stage()
if TREE is None:
    pytest.skip("the reference's sources are not staged (python oracle/stage_ref.py where the tree is mounted)",
                allow_module_level=True)

ORACLE = os.path.dirname(os.path.abspath(stage_ref.__file__))


def test_reference_cli_reproduces_its_pinned_frames(tmp_path):
    r = subprocess.run(["make", "-C", ORACLE, f"REF={TREE}", "-j", str(os.cpu_count() or 4), "_ref/kolmo-ref"],
                       capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    ref = os.path.join(ORACLE, "_ref", "kolmo-ref")
    want = expected_digests(TREE)
    inputs = determinism_inputs(TREE)
    assert len(inputs) == 10
    for name, data in inputs:
        p = str(tmp_path / name)
        open(p, "wb").write(data)
        for level in ("-8", "-9"):
            for t in ("1", "4"):
                z, back = p + ".k", p + ".back"
                subprocess.run([ref, level, "-f", "-T", t, p, "-o", z], check=True, capture_output=True)
                subprocess.run([ref, "-d", "-f", z, "-o", back], check=True, capture_output=True)
                assert open(back, "rb").read() == data, (name, level, t)
                assert hashlib.sha256(open(z, "rb").read()).hexdigest() == want[(name, level)], (name, level, t)
