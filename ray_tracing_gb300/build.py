"""In-tree build of the sm_103a extension, the C++ host library and the oracle.

Everything is compiled with nvcc/g++ directly (no cmake): CUDA sources for
``sm_103a`` only, host sources as C++23. Objects go to ``_build/``; the shared
libraries land next to the code that loads them:

* ``ray_tracing_gb300/_lib/librtgb.so`` — the product (C ABI of ``include/rtgb.h``)
* ``ray_tracing_gb300/_bin/``            — render_realtime, render_restir_acceptance and
  benchmark_scene_lifecycle (C ABI users)
* ``oracle/_bin/liborc.so``             — the CPU oracle (test infrastructure)

Translation units compile in parallel and are skipped when up to date.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "ray_tracing_gb300"
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = ROOT / "_build"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "librtgb.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_bin" / "liborc.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: every a*b+c rounds twice, exactly like the -ffp-contract=off
# oracle; the BVH box test uses explicit fmaf where contraction is wanted.
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++20", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-O2", "-std=c++23", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")


def build_product(jobs: int | None = None, verbose: bool = False) -> Path:
    cuda = _cuda_home()
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "rtgb.h"]
    steps = []
    objects = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objects.append(obj)
        if _stale(obj, [src] + headers):
            steps.append(["nvcc", *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".cpp.o")
        objects.append(obj)
        if _stale(obj, [src] + headers):
            steps.append(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(cuda / "include"),
                          "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for cmd in steps:
            if verbose:
                print(" ".join(cmd))
        list(ex.map(_run, steps))
    if steps or _stale(LIB, objects):
        _run(["nvcc", *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objects),
              "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"])
    return LIB


def build_oracle() -> Path:
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    srcs = [ORACLE_DIR / "radiance_oracle.cpp", ORACLE_DIR / "openpbr_kat.cpp"]
    deps = srcs + [ORACLE_DIR / "oracle_math.h", INCLUDE / "rtgb.h", CSRC / "openpbr.h"]
    if _stale(ORACLE_LIB, deps):
        _run(["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              "-I", str(INCLUDE), "-I", str(CSRC), *map(str, srcs), "-o", str(ORACLE_LIB), "-lpthread"])
    return ORACLE_LIB


CLI_SRC = CSRC / "cli" / "render_realtime.cpp"
CLI = PKG / "_bin" / "render_realtime"
LIFECYCLE_SRC = CSRC / "cli" / "benchmark_scene_lifecycle.cpp"
LIFECYCLE = PKG / "_bin" / "benchmark_scene_lifecycle"
ACCEPTANCE_SRC = CSRC / "cli" / "render_restir_acceptance.cpp"
ACCEPTANCE = PKG / "_bin" / "render_restir_acceptance"


def build_cli() -> Path:
    """The render_realtime CLI and the scene-lifecycle benchmark (C++23 over the
    C ABI), linked against librtgb.so."""
    CLI.parent.mkdir(exist_ok=True)
    deps = [CLI_SRC, CSRC / "cli" / "benchmark_report.h", CSRC / "cli" / "png_writer.h", CSRC / "cli" / "exr_writer.h",
            INCLUDE / "rtgb.h", LIB]
    if _stale(CLI, deps):
        rev = "unknown"
        try:
            rev = subprocess.run(["git", "-C", str(ROOT), "rev-parse", "HEAD"], capture_output=True, text=True,
                                 timeout=10).stdout.strip() or "unknown"
        except (OSError, subprocess.SubprocessError):
            pass
        _run(["g++", *CXX_FLAGS, f"-DRTGB_SOURCE_REVISION=\"{rev}\"", "-I", str(INCLUDE), "-I", str(CSRC / "cli"),
              str(CLI_SRC), "-L", str(LIB_DIR), "-lrtgb", "-Wl,-rpath,$ORIGIN/../_lib", "-o", str(CLI)])
    if _stale(ACCEPTANCE, [ACCEPTANCE_SRC, CSRC / "cli" / "png_reader.h", CSRC / "cli" / "png_writer.h", INCLUDE / "rtgb.h",
                           LIB]):
        _run(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC / "cli"), str(ACCEPTANCE_SRC), "-L", str(LIB_DIR),
              "-lrtgb", "-Wl,-rpath,$ORIGIN/../_lib", "-o", str(ACCEPTANCE)])
    if _stale(LIFECYCLE, [LIFECYCLE_SRC, INCLUDE / "rtgb.h", LIB]):
        _run(["g++", *CXX_FLAGS, "-I", str(INCLUDE), str(LIFECYCLE_SRC), "-L", str(LIB_DIR), "-lrtgb",
              "-Wl,-rpath,$ORIGIN/../_lib", "-o", str(LIFECYCLE)])
    return CLI


def build_all(verbose: bool = False) -> None:
    build_product(verbose=verbose)
    build_cli()
    build_oracle()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
