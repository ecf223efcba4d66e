"""Builds the CUDA library in-tree: particleisosurface_gb300/_lib/libpisurf.so.

Each translation unit is compiled by nvcc for sm_103a only, in parallel, then
linked as a shared library with a C ABI (include/pisurf.h).  Host code is
compiled with -ffp-contract=off so that the host-side float expressions that
mirror the reference (grid bounds, octree root, iso value) round the same way
on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libpisurf.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["sort.cu", "grid.cu", "aniso.cu", "field.cu", "octree.cu", "extract.cu", "api.cu", "noalloc.cu", "qef.cu", "server.cu", "sample.cu", "io.cu", "fp64.cu", "varr.cu", "splash.cu", "h5.cu"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", os.path.join(HERE, "..", "include")]


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(OUT, "obj", src.replace(".cu", ".o"))
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + _flags()
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    if os.path.getmtime(os.path.join(HERE, "..", "include", "pisurf.h")) > t:
        return True
    return False


def build(force=False, verbose_ptxas=False):
    if not force and not _stale():
        return LIB
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in res]
    if verbose_ptxas:
        for (_, log), s in zip(res, SOURCES):
            sys.stderr.write("== %s\n%s" % (s, log))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(force=force, verbose_ptxas="-v" in sys.argv))
