"""The reference's determinism check as data: its seeded inputs and its pinned frame digests, read from the staged
reference tree (benchmark/determinism/check.py runs the whole check when imported, so only its `inputs()` generator
is taken out of it and run)."""
import ast
import os
import random
import struct


def determinism_inputs(tree: str):
    """[(name, bytes)] of the reference's determinism generator."""
    path = os.path.join(tree, "benchmark", "determinism", "check.py")
    mod = ast.parse(open(path).read(), path)
    fn = next(n for n in mod.body if isinstance(n, ast.FunctionDef) and n.name == "inputs")
    ns = {"random": random, "struct": struct}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), path, "exec"), ns)
    return [(name, data) for name, data, _ in ns["inputs"]()]


def expected_digests(tree: str):
    """{(input name, settings): SHA-256 of the frame} from the reference's expected.sha256."""
    out = {}
    for line in open(os.path.join(tree, "benchmark", "determinism", "expected.sha256")):
        parts = line.rstrip("\n").split("  ")
        if len(parts) == 3:
            out[(parts[1], parts[2])] = parts[0]
    return out
