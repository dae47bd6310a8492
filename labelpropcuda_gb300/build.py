"""In-tree build of the GB300 DynLP library (no cmake, no setuptools).

    python -m labelpropcuda_gb300.build          # the library
    python -m labelpropcuda_gb300.build --verbose-ptxas

Produces labelpropcuda_gb300/_build/libdynlp_gb300.so (C ABI, include/dlp_gb300.h
plus the reference-signature C++ shims). Device code is compiled for sm_103a only.
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
INCLUDE = ROOT / "include"
LIB = BUILD / "libdynlp_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    f"-I{INCLUDE}", f"-I{CSRC}",
] + os.environ.get("DLP_NVCC_EXTRA", "").split()  # e.g. -DDLP_SOLO_LANES=8 (build-time tuning)
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-I/usr/local/cuda/include",
             f"-I{INCLUDE}", f"-I{CSRC}"]

CU_SOURCES = ["api.cu", "engine.cu", "engine_kernel.cu", "launchers.cu", "server.cu", "tune.cu"]
CXX_SOURCES = ["host/generate.cpp", "host/problem_cache.cpp", "shims.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    out = (res.stdout + res.stderr).strip()
    if out and os.environ.get("DLP_BUILD_LOG"):
        print(out)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.h")) + list(INCLUDE.glob("*.h")))


def build(verbose_ptxas: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = BUILD / (Path(src).stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            extra = ["-Xptxas", "-v"] if verbose_ptxas else []
            jobs.append([nvcc, *NVCC_FLAGS, *extra, "-c", str(s), "-o", str(o)])
    for src in CXX_SOURCES:
        s = CSRC / src
        if not s.exists():
            continue
        o = BUILD / (Path(src).stem + ".cpp.o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([cxx, *CXX_FLAGS, "-I/usr/local/cuda/include", "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"])
    return LIB


def main(argv: list[str]) -> int:
    lib = build(verbose_ptxas="--verbose-ptxas" in argv, force="--force" in argv)
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
