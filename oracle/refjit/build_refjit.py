"""Build recipe for the reference's own draw-path routines, run on the host CPU.

Test infrastructure only (never part of the product or its timed path).

SwiftShader's draw routines (SetupRoutine, SamplerCore, QuadRasterizer +
PixelRoutine) are Reactor code: C++ that emits IR at run time and JIT-compiles
it.  This script compiles, straight from the read-only reference sources and
with plain gcc/g++ calls (no cmake, no code generation step), everything those
routines need, and links them with this repository's driver of them:

* Subzero (``third_party/subzero``) and its LLVM support subset
  (``third_party/llvm-subzero``, whose generated headers are checked in), the
  x86-64 target: Reactor's second JIT backend (``REACTOR_BACKEND=Subzero``);
* Reactor with that backend (``src/Reactor``: the common files plus
  ``SubzeroReactor.cpp`` and ``Optimizer.cpp``);
* marl (``third_party/marl``), which Reactor's coroutine support links;
* the pipeline / device sources of the routines;
* ``oracle/refjit/refjit_harness.cpp``, which calls the routines directly,
  never through a Vulkan entry point.

The reference's default backend, LLVM 16 (``third_party/llvm-16.0``), does not
build this way: its checked-in tablegen output has no X86 instruction tables
(``configs/common/lib/Target/X86`` lacks ``X86GenInstrInfo.inc``,
``X86GenDAGISel.inc``, ``X86GenMCCodeEmitter.inc`` ...), which only running
llvm-tblgen would generate; ``--stage llvm`` keeps that attempt reproducible.
The one arithmetic difference between the backends on the routines pinned here
is ``MulAdd``: LLVM emits ``llvm.fmuladd`` (fused on FMA hosts), Subzero a
multiply and an add (``SubzeroReactor.cpp`` ``MulAdd``).

Everything it writes goes under ``oracle/_ref/`` (git-ignored); the result is
``oracle/_ref/librefjit.so``.  ``tests/golden/make_refjit_fixtures.py`` calls it
to write the routine-level golden fixtures.  Subzero has no AArch64 target, so
the library is built and run in the x86-64 development container only.

Usage: ``python oracle/refjit/build_refjit.py [--stage subzero,marl,reactor,pipeline,link] [-j N]``
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys
from pathlib import Path

REF = Path(os.environ.get("SWGB_REFERENCE_ROOT", "/root/reference"))
HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
OBJ = OUT / "obj"

LLVM = REF / "third_party" / "llvm-16.0"
LLVM_DIR = LLVM / "llvm"
CFG = LLVM / "configs"

LLVM_INCLUDES = [
    CFG / "linux" / "include",
    LLVM_DIR / "include",
    LLVM_DIR / "lib" / "Target" / "X86",
    CFG / "common" / "include",
    CFG / "common" / "lib" / "IR",
    CFG / "common" / "lib" / "Target" / "X86",
    CFG / "common" / "lib" / "Transforms" / "InstCombine",
    CFG / "common" / "lib" / "ExecutionEngine" / "JITLink",
]
LLVM_FLAGS = [
    "-D__STDC_CONSTANT_MACROS", "-D__STDC_LIMIT_MACROS",
    "-DBLAKE3_NO_AVX512", "-DBLAKE3_NO_AVX2", "-DBLAKE3_NO_SSE41",
    "-DBLAKE3_NO_SSE2", "-DBLAKE3_USE_NEON=0",
    "-Wno-noexcept-type", "-Wno-maybe-uninitialized", "-Wno-deprecated-declarations",
    "-Wno-missing-template-keyword", "-Wno-missing-braces", "-Wno-class-memaccess",
    "-Wno-attributes", "-Wno-init-list-lifetime",
]

COMMON = ["-fPIC", "-O1", "-g0", "-w"]

REACTOR_SRCS = [
    "Assert.cpp", "Debug.cpp", "ExecutableMemory.cpp", "Pragma.cpp", "Reactor.cpp",
    "ReactorDebugInfo.cpp", "SIMD.cpp", "CPUID.cpp", "Optimizer.cpp", "SubzeroReactor.cpp",
]

SUBZERO = REF / "third_party" / "subzero"
LLVM_SZ = REF / "third_party" / "llvm-subzero"
SUBZERO_DEFS = [
    "-DSZTARGET=X8664", "-DALLOW_DUMP=0", "-DALLOW_TIMERS=0", "-DALLOW_LLVM_CL=0", "-DALLOW_LLVM_IR=0",
    "-DALLOW_LLVM_IR_AS_INPUT=0", "-DALLOW_MINIMAL_BUILD=0", "-DALLOW_WASM=0", "-DICE_THREAD_LOCAL_HACK=0",
]
SUBZERO_INCLUDES = [SUBZERO, SUBZERO / "pnacl-llvm" / "include", LLVM_SZ / "include",
                    LLVM_SZ / "build" / "Linux" / "include"]


def cmake_list(path: Path, var: str, cond: str | None = None) -> list[str]:
    """File names listed in a set()/list(APPEND) of one CMakeLists.txt (read as text)."""
    text = path.read_text()
    if cond is None:
        m = re.search(r"set\(" + var + r"\n(.*?)\n\s*\)", text, re.S)
    else:
        m = re.search(re.escape(cond) + r"\)\n\s*list\(APPEND " + var + r"\n(.*?)\n\s*\)", text, re.S)
    out = []
    for line in m.group(1).splitlines():
        line = line.strip().strip('"')
        if line and (line.endswith(".cpp") or line.endswith(".c")):
            out.append(line)
    return out


def subzero_sources() -> list[Path]:
    cm = SUBZERO / "CMakeLists.txt"
    files = cmake_list(cm, "SUBZERO_SRC_FILES") + cmake_list(cm, "SUBZERO_SRC_FILES", 'if(ARCH STREQUAL "x86_64"')
    return [SUBZERO / f for f in files]


def llvm_subzero_sources() -> list[Path]:
    return [LLVM_SZ / f for f in cmake_list(LLVM_SZ / "CMakeLists.txt", "LLVM_SUBZERO_SRC_FILES")]


def llvm_sources() -> list[Path]:
    """The LLVM 16 file list the reference vendors, common part plus x86-64."""
    text = (LLVM / "CMakeLists.txt").read_text()
    common = re.search(r"set\(LLVM_LIST\n(.*?)\n\)", text, re.S).group(1)
    x86 = re.search(
        r'if\(ARCH STREQUAL "x86" OR ARCH STREQUAL "x86_64"\)\n\s*list\(APPEND LLVM_LIST\n(.*?)\n\s*\)',
        text, re.S).group(1)
    files = []
    for line in (common + "\n" + x86).splitlines():
        line = line.strip()
        if line:
            files.append(Path(line.replace("${LLVM_DIR}", str(LLVM_DIR))))
    return files


def marl_sources() -> list[Path]:
    src = REF / "third_party" / "marl" / "src"
    files = [p for p in sorted(src.glob("*.c")) + sorted(src.glob("*.cpp")) + sorted(src.glob("*.S"))
             if "_test" not in p.name and "_bench" not in p.name and "emscripten" not in p.name]
    return files


def compile_one(src: Path, obj: Path, flags: list[str]) -> tuple[Path, str | None]:
    if obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime:
        return obj, None
    obj.parent.mkdir(parents=True, exist_ok=True)
    if src.suffix == ".c":
        cmd = ["gcc", "-std=gnu11"] + COMMON + flags + ["-c", str(src), "-o", str(obj)]
    elif src.suffix == ".S":
        cmd = ["gcc"] + COMMON + flags + ["-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", "-std=c++17"] + COMMON + flags + ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, " ".join(cmd) + "\n" + r.stderr[-4000:]
    return obj, None


def build_stage(name: str, srcs: list[Path], root: Path, flags: list[str], jobs: int) -> Path:
    objs = []
    errors = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = []
        for s in srcs:
            rel = s.relative_to(root)
            obj = OBJ / name / rel.with_suffix(rel.suffix + ".o")
            futs.append(ex.submit(compile_one, s, obj, flags))
        for i, f in enumerate(cf.as_completed(futs)):
            obj, err = f.result()
            objs.append(obj)
            if err:
                errors.append(err)
                print(err, file=sys.stderr)
            if (i + 1) % 100 == 0:
                print(f"[{name}] {i + 1}/{len(srcs)}", flush=True)
    if errors:
        raise SystemExit(f"[{name}] {len(errors)} compile error(s)")
    lib = OUT / f"lib{name}.a"
    if lib.exists():
        lib.unlink()
    subprocess.run(["ar", "rcs", str(lib)] + [str(o) for o in sorted(objs)], check=True)
    print(f"[{name}] {len(objs)} objects -> {lib}", flush=True)
    return lib


def reactor_flags() -> list[str]:
    inc = [REF / "src", REF / "src" / "Reactor", REF / "third_party" / "marl" / "include"] + SUBZERO_INCLUDES
    return ["-I" + str(p) for p in inc] + SUBZERO_DEFS + ["-DREACTOR_ANONYMOUS_MMAP_NAME=swiftshader_jit"]


PIPELINE_SRCS = [
    "Pipeline/SetupRoutine.cpp", "Pipeline/SamplerCore.cpp", "Pipeline/Constants.cpp",
    "Pipeline/ShaderCore.cpp", "Pipeline/PixelRoutine.cpp", "Pipeline/PixelProgram.cpp",
    "Device/QuadRasterizer.cpp", "Device/Clipper.cpp", "Vulkan/VkFormat.cpp",
    "Pipeline/SpirvShader.cpp",
    "System/Half.cpp", "System/Math.cpp", "System/Debug.cpp", "System/Memory.cpp",
]


def pipeline_flags() -> list[str]:
    inc = [REF / "src", REF / "include", REF / "src" / "Reactor",
           REF / "third_party" / "marl" / "include",
           REF / "third_party" / "SPIRV-Headers" / "include",
           REF / "third_party" / "SPIRV-Tools" / "include",
           HERE.parent.parent / "include"]
    return ["-I" + str(p) for p in inc]


def link() -> Path:
    """librefjit.so: the harness, the pipeline objects and the static
    libraries, with every symbol the routines reference resolved at link time
    (-z defs) except those of classes the harness never constructs, which are
    listed by the linker and fail loudly if reached."""
    so = OUT / "librefjit.so"
    libs = [OUT / "libpipeline.a", OUT / "libreactor.a", OUT / "libsubzero.a", OUT / "libllvmsz.a", OUT / "libmarl.a"]
    harness_obj = OBJ / "harness" / "refjit_harness.o"
    objs = sorted((OBJ / "pipeline").rglob("*.o"))
    cmd = (["g++", "-shared", "-o", str(so), str(harness_obj)] + [str(o) for o in objs] +
           ["-Wl,--start-group"] + [str(l) for l in libs if l.exists() and "pipeline" not in l.name] +
           ["-Wl,--end-group", "-lpthread", "-ldl"])
    subprocess.run(cmd, check=True)
    print(f"[link] -> {so}", flush=True)
    return so


def available() -> bool:
    """True where this recipe can run: the reference sources are present and
    the host is x86-64 (Subzero's JIT target)."""
    import platform
    return REF.is_dir() and platform.machine() in ("x86_64", "AMD64")


def main(argv: list[str] | None = None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--stage", default="all")
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args(argv)
    if not REF.exists():
        raise SystemExit(f"reference sources not found at {REF}")
    OUT.mkdir(parents=True, exist_ok=True)
    stages = (["subzero", "marl", "reactor", "pipeline", "harness", "link"] if a.stage == "all"
              else a.stage.split(","))
    if "subzero" in stages:
        flags = ["-I" + str(p) for p in SUBZERO_INCLUDES] + SUBZERO_DEFS
        build_stage("llvmsz", llvm_subzero_sources(), LLVM_SZ, flags, a.j)
        build_stage("subzero", subzero_sources(), SUBZERO, flags, a.j)
    if "llvm" in stages:
        build_stage("llvm16", llvm_sources(), LLVM_DIR,
                    ["-I" + str(p) for p in LLVM_INCLUDES] + LLVM_FLAGS, a.j)
    if "marl" in stages:
        m = REF / "third_party" / "marl"
        build_stage("marl", marl_sources(), m / "src", ["-I" + str(m / "include")], a.j)
    if "reactor" in stages:
        srcs = [REF / "src" / "Reactor" / f for f in REACTOR_SRCS]
        build_stage("reactor", srcs, REF / "src" / "Reactor", reactor_flags(), a.j)
    if "pipeline" in stages:
        srcs = [REF / "src" / f for f in PIPELINE_SRCS]
        build_stage("pipeline", srcs, REF / "src", pipeline_flags(), a.j)
    if "harness" in stages:
        obj, err = compile_one(HERE / "refjit_harness.cpp", OBJ / "harness" / "refjit_harness.o",
                               pipeline_flags() + ["-Wall"])
        if err:
            raise SystemExit(err)
    if "link" in stages:
        link()


if __name__ == "__main__":
    main()
