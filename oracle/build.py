"""TEST INFRASTRUCTURE ONLY — builds the CPU oracle (oracle/_build/libcostal_oracle.so).

The oracle restates the reference's CPU algorithms in C++ (costal_oracle.cpp, oracle_tile.cpp).
It is compiled with g++ only, with -ffp-contract=off except for the coarse tile product, and with
no architecture-specific flags, so it builds and gives the same results on x86_64 and aarch64.

The reference itself (Rust, crates/costal-core) cannot be compiled here: there is no cargo/rustc,
so there is no oracle/_ref build; parity is pinned through the reference's own known answers and
golden digests instead (see costal_oracle.cpp's header).
"""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libcostal_oracle.so"
SOURCES = [HERE / "costal_oracle.cpp", HERE / "oracle_tile.cpp"]
COMMON = ["-O3", "-std=c++17", "-fPIC", "-fopenmp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    inputs = SOURCES + [Path(__file__)]
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in inputs):
        return LIB
    objs = []
    for src, contract in ((SOURCES[0], "off"), (SOURCES[1], "fast")):
        obj = BUILD / (src.stem + ".o")
        _run(["g++", *COMMON, f"-ffp-contract={contract}", "-c", str(src), "-o", str(obj)])
        objs.append(str(obj))
    tmp = BUILD / "libcostal_oracle.so.tmp"
    _run(["g++", "-shared", "-fopenmp", "-o", str(tmp), *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
