"""Builds the in-tree CUDA library libpagani_gb300.so for sm_103a.

Translation units are compiled in parallel with nvcc and linked into one
shared object next to this file.  The device code is compiled with
--fmad=false (every fused multiply-add is explicit in the source) and the host
code with -ffp-contract=off, so results do not depend on the host compiler's
contraction defaults (aarch64 GCC contracts by default, x86-64 does not).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpagani_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["pg_rule.cpp", "pg_engine.cu", "pg_capi.cu", "pg_mcubes.cu", "pg_noalloc.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit to build")
    return exe


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I" + os.path.join(HERE, "..", "include")] + ARCH


def _compile(src):
    out = os.path.join(BUILD, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "pagani_gb300.h")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    lang = ["-x", "cu"]
    cmd = [nvcc()] + _flags() + lang + ["-c", path, "-o", out]
    subprocess.check_call(cmd)
    return out


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    subprocess.check_call(cmd)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
