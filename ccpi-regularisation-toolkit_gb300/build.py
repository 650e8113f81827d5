"""Build the GB300 regulariser libraries in-tree.

Compiles every ``csrc/*.cu`` for sm_103a (one ``-gencode``, translation units
in parallel) and links, under ``ccpi/filters/``, the two names the
reference's Python layer loads (src/Python/ccpi/filters/utils.py:62-68):

* ``libcilregcuda.so`` — every entry point of ``include/cilreg_gb300.h``: the
  ``*_GPU_main`` and ``*_CPU_main`` families (all executing on the GPU) and
  the device-pointer API;
* ``libcilreg.so``     — a small C library exporting the same entry points,
  each forwarding to ``libcilregcuda.so`` (opened beside it), so that a
  process loading both holds one CUDA runtime, one launch counter and one
  copy of every device array.  Its source is generated from the header.

Usage: ``python build.py [--force]``.  Objects go to ``_build/`` (ignored by git).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "ccpi", "filters")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

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


def _prototypes():
    """(return type, name, parameter list, argument names) of every function
    the public header declares."""
    text = open(os.path.join(INCLUDE, "cilreg_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M).replace('extern "C" {', "")
    out = []
    for decl in re.sub(r"\s+", " ", text).split(";"):
        m = re.fullmatch(r"\s*([A-Za-z_][A-Za-z0-9_ ]*?[ *]+)([A-Za-z_][A-Za-z0-9_]*)\((.*)\)\s*", decl)
        if not m:
            continue
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
        names = [] if params in ("", "void") else [re.findall(r"[A-Za-z_][A-Za-z0-9_]*", q)[-1]
                                                   for q in params.split(",")]
        out.append((ret, name, params, names))
    return out


def forwarding_source() -> str:
    """C source of libcilreg.so: each header entry point forwards to the
    definition in libcilregcuda.so, resolved once when the library loads."""
    lines = ["/* generated by build.py from include/cilreg_gb300.h: forwards every entry point",
             " * to libcilregcuda.so in the same directory (one copy of the GPU library per",
             " * process) */",
             "#define _GNU_SOURCE", "#include <dlfcn.h>", "#include <stdio.h>", "#include <string.h>",
             '#include "cilreg_gb300.h"', "", "static void *g_impl;", ""]
    protos = _prototypes()
    for ret, name, params, names in protos:
        fail = '"libcilregcuda.so could not be loaded"' if "char" in ret else f"({ret})-3"
        lines += [f"static {ret} (*p_{name})({params});",
                  f"{ret} {name}({params}) {{",
                  f"    if (!p_{name}) return {fail};",
                  f"    return p_{name}({', '.join(names)});", "}", ""]
    lines += ["__attribute__((constructor)) static void cilreg_forward_init(void) {",
              "    Dl_info info;",
              "    char path[4096];",
              "    if (!dladdr((void *)&cilreg_forward_init, &info) || !info.dli_fname) return;",
              "    strncpy(path, info.dli_fname, sizeof(path) - 32);",
              "    path[sizeof(path) - 32] = 0;",
              "    char *slash = strrchr(path, '/');",
              "    strcpy(slash ? slash + 1 : path, \"libcilregcuda.so\");",
              "    g_impl = dlopen(path, RTLD_NOW | RTLD_LOCAL);",
              "    if (!g_impl) {",
              '        fprintf(stderr, "libcilreg: cannot load %s: %s\\n", path, dlerror());',
              "        return;", "    }"]
    for ret, name, params, names in protos:
        lines.append(f'    *(void **)&p_{name} = dlsym(g_impl, "{name}");')
    lines += ["}", ""]
    return "\n".join(lines)


def build(force: bool = False, verbose: bool = True) -> list:
    os.makedirs(OBJ, exist_ok=True)
    hdr = _deps()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, hdr), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    gpu_lib = os.path.join(OUT, "libcilregcuda.so")
    if force or not os.path.exists(gpu_lib) or os.path.getmtime(gpu_lib) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", gpu_lib] + objs + ["-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed for libcilregcuda.so:\n{r.stdout}\n{r.stderr}")
    fwd_src = os.path.join(OBJ, "cilreg_forward.c")
    src = forwarding_source()
    if not os.path.exists(fwd_src) or open(fwd_src).read() != src:
        with open(fwd_src, "w") as f:
            f.write(src)
    cpu_lib = os.path.join(OUT, "libcilreg.so")
    if force or not os.path.exists(cpu_lib) or os.path.getmtime(cpu_lib) < os.path.getmtime(fwd_src):
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-Wall", "-I", INCLUDE, "-o", cpu_lib, fwd_src,
               "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed for libcilreg.so:\n{r.stdout}\n{r.stderr}")
    outs = [gpu_lib, cpu_lib]
    if verbose:
        print("built", ", ".join(os.path.relpath(p, HERE) for p in outs))
    return outs


if __name__ == "__main__":
    build(force="--force" in sys.argv)
