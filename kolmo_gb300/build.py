"""In-tree build of the native parts: the CUDA library behind the C ABI (``libkgbwt.so``, sm_103a only) and the
host-only workload generators (``libkgbwt_workloads.so``). Translation units compile in parallel; nothing is
installed outside the package directory."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_native")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["fwd.cu", "inv.cu", "api.cu", "serve.cu"]
LIB = os.path.join(OUT, "libkgbwt.so")
LIB_CHECKED = os.path.join(OUT, "libkgbwt_checked.so")
WORKLOADS = os.path.join(OUT, "libkgbwt_workloads.so")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_workloads(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, "workloads.c")
    if force or not _newer(WORKLOADS, [src]):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", WORKLOADS, src])
    return WORKLOADS


def build_cuda(force: bool = False, extra: list[str] | None = None, verbose_ptxas: bool = False,
               checked: bool = False) -> str:
    """Compiles the CUDA library; checked=True builds the bounds-checked variant (every guarded device write is
    range-checked and reports an error bit instead of touching memory) as libkgbwt_checked.so."""
    os.makedirs(OUT, exist_ok=True)
    suffix = "_checked" if checked else ""
    lib = LIB_CHECKED if checked else LIB
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "kgbwt.h"))
    objs = []
    jobs = []
    for unit in CUDA_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT, unit.replace(".cu", suffix + ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
                   "-c", src, "-o", obj]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            if checked:
                cmd.append("-DKGB_CHECKED")
            cmd += extra or []
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=len(CUDA_UNITS)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not _newer(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart", "-lpthread", "-ldl"])
    return lib


def build_all(force: bool = False, checked: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        fs = [ex.submit(build_cuda, force), ex.submit(build_workloads, force)]
        if checked:
            fs.append(ex.submit(build_cuda, force, None, False, True))
        for f in fs:
            f.result()


if __name__ == "__main__":
    import sys

    build_all(force="-f" in sys.argv, checked="--checked" in sys.argv)
    print(LIB)
