"""Loads tests/golden/bwt_golden.json (hashes of the reference sorter's outputs, made by tests/golden/make_golden.py)
and regenerates each case's input with kolmo_gb300.workloads."""
import json
import os

import numpy as np

from kolmo_gb300 import workloads as W
import refgen as R

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "bwt_golden.json")) as f:
        return json.load(f)["cases"]


def make_input(c) -> np.ndarray:
    g = c["gen"]
    if g == "test_block":
        return R.test_block(c["kind"], c["n"])
    if g == "markov_1mib":
        return W.markov_1mib()
    if g == "source":
        return W.source_block(c["source"], c["n"], c["seed"])
    if g == "periodic":
        return W.periodic(c["n"], c["seed"], c["period"], c["flip"])
    if g == "fibonacci":
        return W.fibonacci(c["n"])
    if g == "prose":
        return W.zipf_prose(c["n"], c["seed"], ncopies=c["ncopies"])
    raise ValueError(g)


def h(a) -> str:
    return "%016x" % W.fnv1a(np.ascontiguousarray(a))
