"""Builds libttsh.so in-tree (bacterial-droplet_gb300/lib/) with nvcc for sm_103a.

Translation units are compiled in parallel and linked with nvcc; the result is
git-ignored. No cmake, no torch extension machinery: the library is a plain
C-ABI shared object (include/ttsh.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libttsh.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "plain.cu", "fft.cu", "fftreg_f32.cu", "fftreg_f64.cu", "fused.cu", "io.cpp", "noalloc.cu", "post.cu"]


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _deps_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(PKG), "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJDIR, src + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "-c",
           os.path.join(CSRC, src), "-o", obj] + extra
    if src.endswith(".cu"):
        cmd += ARCH + ["--expt-relaxed-constexpr"]
    else:
        cmd = [nvcc(), "-x", "c++"] + cmd[1:]
    subprocess.check_call(cmd)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
