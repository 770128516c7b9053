"""ORACLE -- test infrastructure only: stages the reference's own sources for machines without the reference tree.

The GPU host has no copy of adnaneben/kolmo, and binaries built on this x86 container do not run on its Arm cores.
This script copies the parts of the reference tree that the CPU oracle needs into ``baseline/_ref/kolmo/`` (listed
in ``.gitignore``: never committed, but carried with the working tree to the GPU host), where ``oracle/Makefile``
compiles them:

* ``src/`` -- the sorter (``src/algo/sais/sais.c``, ``src/algo/par.c``) for ``_ref/libkref.so``, and the whole
  library and CLI (``src/kolmo.c``, ``src/cli/``) for the frame-parity binaries ``_ref/kolmo-ref`` and
  ``_ref/kolmo-gpu``;
* ``benchmark/determinism/`` -- the reference's seeded frame generator and its pinned SHA-256 digests;
* ``tests/v12/`` and ``tests/v12.sha256`` -- frames written by reference releases, with the digests of their inputs.

Nothing here is part of the product: only the tests and the CPU-baseline leg of ``bench.py`` use what it stages.

    python oracle/stage_ref.py [REFERENCE_TREE]     # default: $KOLMO_REFERENCE_TREE, else /root/reference
"""
from __future__ import annotations

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGED = os.path.join(ROOT, "baseline", "_ref", "kolmo")
PARTS = ("src", "benchmark/determinism", "tests/v12", "tests/v12.sha256", "VERSION", "LICENSE", "NOTICE")


def source_tree(arg: str | None = None) -> str | None:
    for cand in (arg, os.environ.get("KOLMO_REFERENCE_TREE"), "/root/reference"):
        if cand and os.path.exists(os.path.join(cand, "src", "algo", "sais", "sais.c")):
            return cand
    return None


def staged() -> str | None:
    """The staged tree, or None when nothing was staged on (or carried to) this machine."""
    return STAGED if os.path.exists(os.path.join(STAGED, "src", "algo", "sais", "sais.c")) else None


def _same(a: str, b: str) -> bool:
    try:
        sa, sb = os.stat(a), os.stat(b)
    except OSError:
        return False
    return sa.st_size == sb.st_size and int(sa.st_mtime) == int(sb.st_mtime)


def stage(src: str | None = None) -> str | None:
    """Copies the reference parts into the staging directory (files already there with the same size and time are
    kept). Returns the staged tree, or the existing one when no reference tree is mounted here."""
    tree = source_tree(src)
    if tree is None:
        return staged()
    for part in PARTS:
        s = os.path.join(tree, part)
        if not os.path.exists(s):
            continue
        if os.path.isdir(s):
            for dirpath, _, files in os.walk(s):
                rel = os.path.relpath(dirpath, tree)
                os.makedirs(os.path.join(STAGED, rel), exist_ok=True)
                for f in files:
                    a, b = os.path.join(dirpath, f), os.path.join(STAGED, rel, f)
                    if not _same(a, b):
                        shutil.copy2(a, b)
        else:
            d = os.path.join(STAGED, part)
            os.makedirs(os.path.dirname(d), exist_ok=True)
            if not _same(s, d):
                shutil.copy2(s, d)
    return STAGED


if __name__ == "__main__":
    out = stage(sys.argv[1] if len(sys.argv) > 1 else None)
    print(out or "no reference tree found and nothing staged")
