"""Builds libelgb300.so in-tree (elemental_gb300/lib/) for sm_103a.

Every CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a`` in parallel; host C++ units by
g++; one shared library is linked against the shared CUDA runtime (so a
process that already loaded PyTorch's runtime shares it).  No cmake, no
torch extension machinery: the library has no torch dependency.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libelgb300.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _newest_input():
    ts = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            ts = max(ts, os.path.getmtime(os.path.join(d, f)))
    return ts


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles and links the library if any source is newer; returns its path."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= _newest_input()):
        return LIB
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(OBJDIR, exist_ok=True)
    cu, cpp = sources()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    objs = []
    for f in cu:
        o = os.path.join(OBJDIR, f + ".o")
        objs.append(o)
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-v" if verbose else "-O3", *inc, "-c",
                     os.path.join(CSRC, f), "-o", o])
    for f in cpp:
        o = os.path.join(OBJDIR, f + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-Wall", "-Wno-unused-function",
                     "-I" + os.path.join(home, "include"), *inc, "-c",
                     os.path.join(CSRC, f), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for err in ex.map(_compile, jobs):
            if verbose and err:
                sys.stderr.write(err)
    tmp = LIB + f".tmp{os.getpid()}"
    link = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs,
            "-Xlinker", "-rpath," + os.path.join(home, "lib64")]
    _compile(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
