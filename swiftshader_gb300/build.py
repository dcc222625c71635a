"""Builds libswgb.so in-tree with nvcc for sm_103a.

The library is compiled with -ftz=true -prec-div=true -prec-sqrt=true
-fmad=false: subnormals flush like the reference's FTZ/DAZ worker threads,
divisions are IEEE-rounded, and only the explicit fused multiply-adds of the
kernels (the reference's MulAdd) are fused.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libswgb.so")
SOURCES = [os.path.join(CSRC, "swgb_draw.cu")]
DEPS = SOURCES + [os.path.join(CSRC, "swgb_numeric.cuh"), os.path.join(ROOT, "include", "swgb.h")]

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3", "-std=c++17",
              "-ftz=true", "-prec-div=true", "-prec-sqrt=true", "-fmad=false",
              "-Xcompiler", "-fPIC", "-shared", "-diag-suppress", "177"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in DEPS)


def build(force=False, verbose=False):
    """Compiles the extension if a source is newer than the library."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and up_to_date():
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + NVCC_FLAGS + ["-o", tmp] + SOURCES
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
