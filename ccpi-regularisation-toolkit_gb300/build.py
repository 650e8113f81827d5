"""Build the GB300 regulariser libraries in-tree.

Compiles every ``csrc/*.cu`` for sm_103a (one ``-gencode``, translation units
in parallel) and links two shared libraries with identical contents under
``ccpi/filters/`` — the names the reference's Python layer loads
(src/Python/ccpi/filters/utils.py:62-68):

* ``libcilregcuda.so`` — the ``*_GPU_main`` family and the device-pointer API;
* ``libcilreg.so``     — the ``*_CPU_main`` family (executing on the GPU).

Usage: ``python build.py [--force]``.  Objects go to ``_build/`` (ignored by git).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "ccpi", "filters")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIBS = ("libcilregcuda.so", "libcilreg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-Xptxas", "-O3",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return max((os.path.getmtime(h) for h in headers), default=0.0)


def _compile(src: str, force: bool, hdr_mtime: float) -> str:
    obj = os.path.join(OBJ, src[:-3] + ".o")
    srcp = os.path.join(CSRC, src)
    if not force and os.path.exists(obj):
        if os.path.getmtime(obj) >= max(os.path.getmtime(srcp), hdr_mtime):
            return obj
    cmd = [nvcc()] + NVCC_FLAGS + ["-I", CSRC, "-I", INCLUDE, "-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = True) -> list:
    os.makedirs(OBJ, exist_ok=True)
    hdr = _deps()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, hdr), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    outs = []
    for lib in LIBS:
        path = os.path.join(OUT, lib)
        if force or not os.path.exists(path) or os.path.getmtime(path) < newest:
            cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", path] + objs + ["-lpthread", "-ldl", "-lrt"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed for {lib}:\n{r.stdout}\n{r.stderr}")
        outs.append(path)
    if verbose:
        print("built", ", ".join(os.path.relpath(p, HERE) for p in outs))
    return outs


if __name__ == "__main__":
    build(force="--force" in sys.argv)
