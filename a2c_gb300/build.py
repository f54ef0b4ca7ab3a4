"""Build recipe for liba2c_gpp.so (the C ABI in include/a2c_gpp.h).

Every CUDA translation unit is compiled for sm_103a only, in parallel, into
a2c_gb300/_build/, and linked into a2c_gb300/_lib/liba2c_gpp.so.  The FP64
translation units are compiled with -fmad=false: the plain form reproduces
the reference's arithmetic, which performs every multiply and add
separately.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "liba2c_gpp.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-I", str(ROOT / "include"), "-I", str(CSRC)]
# translation units whose arithmetic must not be contracted into FMA
NO_FMA = {"k_fp64.cu", "k_neighbors.cu", "k_misc.cu", "lbfgs.cu", "batch.cu", "k_lattice.cu"}
CU_SOURCES = ["api.cu", "k_fp64.cu", "k_neighbors.cu", "k_misc.cu", "lbfgs.cu", "k_mixed.cu", "k_peak.cu", "batch.cu", "k_lattice.cu"]
CPP_SOURCES = ["lattice.cpp", "lattice_csg.cpp", "tables.cpp", "host_io.cpp", "snapshot.cpp", "input_reader.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liba2c_gpp")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    nv = nvcc()
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        flags = NVCC_COMMON + (["-fmad=false"] if src in NO_FMA else []) + (extra_flags or [])
        if _stale(o, [s, *headers, Path(__file__)]):
            jobs.append([nv, *flags, "-c", str(s), "-o", str(o)])
    for src in CPP_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if _stale(o, [s, *headers, Path(__file__)]):
            jobs.append(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-I", str(ROOT / "include"),
                         "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, fut in [(j, ex.submit(_run, j)) for j in jobs]:
            fut.result()
            if verbose:
                print(" ".join(cmd))
    if jobs or not LIB.exists():
        _run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
