"""Builds libswgb.so in-tree with nvcc for sm_103a.

Six translation units are compiled in parallel and linked into one library:
swgb_draw.cu (vertex, setup and adjoint kernels, host side, C-ABI),
swgb_blit.cu (clears, resolves, blits) and swgb_raster.cu once per colour
format (the raster kernel variants).

Every unit is compiled with -prec-div=true -prec-sqrt=true -fmad=false
(divisions IEEE-rounded, only the explicit fused multiply-adds of the kernels
-- the reference's MulAdd -- fused) and, except swgb_blit.cu, -ftz=true:
subnormals flush like the reference's FTZ/DAZ worker threads.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libswgb.so")
# (source, extra defines, object name)
# The Blitter unit keeps IEEE subnormals (-ftz=false): the reference runs blit
# routines on its queue thread, which does not set FTZ/DAZ.
UNITS = [("swgb_draw.cu", ["-ftz=true"], "swgb_draw.o"), ("swgb_blit.cu", ["-ftz=false"], "swgb_blit.o")] + [
    ("swgb_raster.cu", ["-ftz=true", "-DSWGB_RASTER_CF=%d" % cf], "swgb_raster_cf%d.o" % cf) for cf in range(4)]
SOURCES = [os.path.join(CSRC, u) for u in ("swgb_draw.cu", "swgb_raster.cu", "swgb_blit.cu")]
DEPS = SOURCES + [os.path.join(CSRC, h) for h in ("swgb_kernels.cuh", "swgb_numeric.cuh", "swgb_adjoint.cuh", "swgb_blit.h",
                                                  "swgb.map")] + \
    [os.path.join(ROOT, "include", "swgb.h")]

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3", "-std=c++17",
              "-prec-div=true", "-prec-sqrt=true", "-fmad=false",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-diag-suppress", "177"]


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
    """Compiles the library if a source is newer than it (units in parallel)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and up_to_date():
        return LIB
    tag = ".tmp%d" % os.getpid()
    procs, objs = [], []
    for src, defs, obj in UNITS:
        o = os.path.join(BUILD, obj[:-2] + tag + ".o")
        cmd = [nvcc()] + NVCC_FLAGS + defs + ["-c", "-o", o, os.path.join(CSRC, src)]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(o)
    failed = [cmd for p, cmd in procs if p.wait() != 0]
    if failed:
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
        raise subprocess.CalledProcessError(1, failed[0])
    tmp = LIB[:-3] + tag + ".so"
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared",
           "-Xlinker", "--version-script=" + os.path.join(CSRC, "swgb.map"), "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    for o in objs:
        os.remove(o)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
