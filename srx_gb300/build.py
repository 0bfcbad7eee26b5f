"""Build of the CUDA library and tools (in-tree, sm_103a only).

``build()`` compiles ``srx_gb300/csrc`` into ``srx_gb300/_lib/libevpg.so``
(the C ABI of ``include/evpg.h``) and ``srx_gb300/_lib/evpg_run`` (the
command-line driver). Translation units are compiled in parallel; outputs are
rebuilt only when a source is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(LIBDIR, "libevpg.so")
RUN = os.path.join(LIBDIR, "evpg_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["evpg_api.cu", "evpg_spectral.cu", "evpg_solver.cu", "evpg_batch.cu"]
C_SOURCES = ["host/evpg_job.c", "host/evpg_serve.c"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list:
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".cu", ".cuh", ".h", ".c"))]
    return out + [os.path.join(INCLUDE, "evpg.h")]


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in _deps())


def _run(cmd: list) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile everything if needed; returns the library path."""
    if not force and not _stale(LIB) and not _stale(RUN):
        return LIB
    nvcc = _nvcc()
    obj = os.path.join(LIBDIR, "obj")
    os.makedirs(obj, exist_ok=True)
    jobs = []
    for s in CU_SOURCES:
        o = os.path.join(obj, os.path.basename(s) + ".o")
        jobs.append([nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-I", INCLUDE, "-c", os.path.join(CSRC, s), "-o", o])
    for s in C_SOURCES + ["host/evpg_run.c"]:
        o = os.path.join(obj, os.path.basename(s) + ".o")
        jobs.append(["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-Wall",
                     "-I", INCLUDE, "-c", os.path.join(CSRC, s), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    objs = [os.path.join(obj, os.path.basename(s) + ".o") for s in CU_SOURCES + C_SOURCES]
    _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lm", "-lpthread"])
    _run([nvcc, *ARCH, "-o", RUN, os.path.join(obj, "evpg_run.c.o"), "-L", LIBDIR, "-levpg",
          "-Xlinker", "-rpath,$ORIGIN", "-lm"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
