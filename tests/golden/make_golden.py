"""Generates tests/golden/bwt_golden.json from the REFERENCE's own suffix sorter.

Run in a checkout where the reference tree is mounted and ``make -C oracle`` has built ``oracle/_ref/libkref.so``
from the reference's src/algo/sais/sais.c and src/algo/par.c. For every case the script records hashes of the
reference's BWT (U), its sampled indexes (I) and the suffix array implied by them (derived by the LF walk, since the
reference exposes no suffix array), plus a hash of the input so that a machine regenerating the input can check it
got the same bytes. Inputs come from kolmo_gb300.workloads and tests/refgen.py (deterministic on every platform).

Cases:
  * the reference's own suffix-sorter test matrix (tests/test_bwt.c:97-121): block kinds 0-8 of its generator, the
    sizes it uses, r in {2, 2^10, 2^19} where (n - 1) / r <= 1000;
  * the benchmark workloads at sizes the CPU sorter finishes in seconds: the 1 MiB order-2 Markov block with the
    codec-18 sampling interval, the three mixed-batch sources, periodic inputs with flips and the Fibonacci word;
  * a few tiny cases stored in full.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle as O  # noqa: E402
from kolmo_gb300 import workloads as W
import refgen as R  # noqa: E402
from kolmo_gb300.host import codec18_rlog  # noqa: E402

TEST_SIZES = [2, 3, 7, 100, 4096, 65536, 70001, 300000, 1000003]


def h(a) -> str:
    return "%016x" % W.fnv1a(np.ascontiguousarray(a))


def case(name: str, T: np.ndarray, r: int, full: bool = False) -> dict:
    rc, U, I = O.bwt_aux(T, r, use_ref=True)
    assert rc == 0, (name, rc)
    SA = O.sa_from_bwt(U, int(I[0])) if T.size > 1 else np.zeros(T.size, np.int32)
    rc2, back = O.unbwt_aux(U, r, I, use_ref=True)
    assert rc2 == 0 and np.array_equal(back, T), name
    d = {"name": name, "n": int(T.size), "r": int(r), "input": h(T), "U": h(U), "I": h(I.astype("<i4")),
         "I0": int(I[0]), "nI": int(I.size), "SA": h(SA.astype("<i4"))}
    if full:
        d["U_hex"] = U.tobytes().hex()
        d["I_list"] = [int(x) for x in I]
        d["T_hex"] = T.tobytes().hex()
    return d


def main() -> None:
    if O.ref_lib() is None:
        raise SystemExit("reference sorter not built (make -C oracle with the reference tree mounted)")
    cases = []
    for kind in range(9):
        for n in TEST_SIZES:
            T = R.test_block(kind, n)
            for rl in (1, 10, 19):
                r = 1 << rl
                if (n - 1) // r > 1000:
                    continue
                cases.append(dict(case(f"test_block/{kind}/{n}/{r}", T, r), gen="test_block", kind=kind))
    T = W.markov_1mib()
    cases.append(dict(case("markov_1mib", T, 1 << codec18_rlog(T.size)), gen="markov_1mib"))
    for src in range(3):
        for n, seed in ((300000, 11), (2 << 20, 12)):
            T = W.source_block(src, n, seed)
            cases.append(dict(case(f"source/{src}/{n}", T, 1 << codec18_rlog(n)), gen="source", source=src,
                              seed=seed))
    for period in (1, 7, 4096):
        n = 1 << 20
        T = W.periodic(n, 99 + period, period, 1 << 18)
        cases.append(dict(case(f"periodic/{period}/{n}", T, 1 << codec18_rlog(n)), gen="periodic", period=period,
                          seed=99 + period, flip=1 << 18))
    T = W.fibonacci(1 << 20)
    cases.append(dict(case("fibonacci/1048576", T, 1 << codec18_rlog(T.size)), gen="fibonacci"))
    T = W.zipf_prose(4 << 20, 77, ncopies=20)
    cases.append(dict(case("prose/4194304", T, 1 << codec18_rlog(T.size)), gen="prose", seed=77, ncopies=20))
    for i, (kind, n, r) in enumerate(((8, 40, 2), (3, 17, 4), (1, 64, 8), (0, 9, 2), (7, 100, 16))):
        T = R.test_block(kind, n)
        cases.append(dict(case(f"tiny/{i}", T, r, full=True), gen="test_block", kind=kind))
    out = {"generator": "tests/golden/make_golden.py", "sorter": "reference src/algo/sais/sais.c (libsais 2.12.1 subset)",
           "hash": "fnv-1a 64", "cases": cases}
    with open(os.path.join(HERE, "bwt_golden.json"), "w") as f:
        json.dump(out, f, indent=0)
    print(f"{len(cases)} cases written")


if __name__ == "__main__":
    main()
