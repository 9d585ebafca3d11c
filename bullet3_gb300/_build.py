"""In-tree build of the CUDA library (libb3gpu.so).

The CUDA translation units are compiled for sm_103a only, in parallel, with --fmad=false so the
physics kernels follow the same IEEE operation sequence as the oracle.  Rebuilds only when a
source is newer than the shared object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libb3gpu.so"

CU_SOURCES = ["primitives.cu", "broadphase.cu", "narrowphase.cu", "solver.cu", "integrate.cu", "world.cu",
              "noalloc.cu", "mlp.cu", "warmstart.cu", "primitives_capi.cu", "raycast.cu", "joints.cu"]
CPP_SOURCES = ["hull.cpp"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libb3gpu.so")


def _newer(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build command failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def build_library(force: bool = False, verbose: bool = False) -> Path:
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    sources = [CSRC / s for s in CU_SOURCES + CPP_SOURCES]
    if not force and not _newer(LIB, sources + headers):
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + str(ROOT / "include"), "-I" + str(CSRC)]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = BUILD / (s + ".o")
        objs.append(o)
        if force or _newer(o, [CSRC / s] + headers):
            jobs.append([nvcc, ARCH] + common + ["-c", str(CSRC / s), "-o", str(o)])
    for s in CPP_SOURCES:
        o = BUILD / (s + ".o")
        objs.append(o)
        if force or _newer(o, [CSRC / s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I" + str(ROOT / "include"),
                         "-I" + str(CSRC), "-c", str(CSRC / s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, ARCH, "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
