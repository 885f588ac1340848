"""Build libcostal_gb300.so in-tree: nvcc for the sm_103a kernels, g++ for the host Leiden.

    python -m costal_gb300.build            # or costal_gb300.build.build_library()

Every CUDA translation unit is compiled for `-gencode arch=compute_103a,code=sm_103a` only, in
parallel, into costal_gb300/_build/. Host code is compiled with -ffp-contract=off: the host Leiden
and the host halves of the .cu files must never fuse a multiply and an add (the reference, in
Rust, never does). No architecture-specific host flags, so the same recipe builds on x86_64 and on
the aarch64 (Grace) host of a GB300.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libcostal_gb300.so"
INCLUDE = ROOT / "include"

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp",
    f"-I{INCLUDE}", f"-I{CSRC}",
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcostal_gb300")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    deps = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, deps


def _stale(target: Path, inputs) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build_library(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile every kernel and host source into costal_gb300/_build/libcostal_gb300.so."""
    cu, cpp, deps = _sources()
    BUILD.mkdir(exist_ok=True)
    if not force and not ptxas_info and not _stale(LIB, cu + cpp + deps + [Path(__file__)]):
        return LIB
    nvcc = _nvcc()
    jobs = []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        flags = NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + os.environ.get("COSTAL_NVCC_EXTRA", "").split()
        jobs.append([nvcc, *flags, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD / (src.stem + ".cpp.o")
        jobs.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for log in logs:
            if log.strip():
                print(log, file=sys.stderr)
    objs = [str(BUILD / (s.stem + ".cu.o")) for s in cu] + [str(BUILD / (s.stem + ".cpp.o")) for s in cpp]
    tmp = BUILD / (LIB.name + ".tmp")
    _run([nvcc, *GENCODE, "-shared", "-o", str(tmp), *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
