"""Builds liblgame_gpu.so (CUDA kernels for sm_103a + the C ABI + the host set-up) in-tree.

Translation units are compiled in parallel with nvcc / g++ and linked with the static
CUDA runtime, so the library only needs the driver at run time.  The FP64 kernels are
compiled with -fmad=false: the FP64 step keeps every multiply and add separately
rounded, as the reference's arithmetic is written, which makes it bitwise comparable
with the CPU oracle.  Output: l-game_gb300/_build/liblgame_gpu.so
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "liblgame_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               f"-I{ROOT / 'include'}", f"-I{CSRC}", "--expt-relaxed-constexpr"]
CXX_COMMON = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-fopenmp",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]

# (source, extra flags)
CUDA_UNITS = [
    ("lgame_gpu.cu", ["-fmad=false"]),
    ("kernels_fp64.cu", ["-fmad=false"]),
    ("column_fp64.cu", ["-fmad=false"]),
    ("split.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
    ("emulator.cu", []),
]
CXX_UNITS = [
    ("host/error.cpp", []),
    ("host/namelist.cpp", []),
    ("host/setup.cpp", []),
    ("host/teacher.cpp", []),
    ("host/files.cpp", []),
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return [CSRC / s for s, _ in CUDA_UNITS + CXX_UNITS] + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) \
        + sorted((ROOT / "include").glob("*.h")) + [Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources() if p.exists())


def _run(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, p.returncode, p.stdout + p.stderr


def build(verbose: bool = False, force: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src, flags in CUDA_UNITS:
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        jobs.append([nvcc, *ARCH, *NVCC_COMMON, *flags, "-c", str(CSRC / src), "-o", str(obj)])
    for src, flags in CXX_UNITS:
        obj = OUT / (Path(src).stem + ".host.o")
        objs.append(obj)
        jobs.append(["g++", *CXX_COMMON, *flags, "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for cmd, rc, out in ex.map(_run, jobs):
            if verbose or rc != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + out)
            if rc != 0:
                raise RuntimeError(f"compilation failed: {' '.join(cmd[-3:])}")
    tmp = OUT / "liblgame_gpu.so.tmp"
    cmd, rc, out = _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static",
                         "-Xcompiler", "-fopenmp"])
    if verbose or rc != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + out)
    if rc != 0:
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
