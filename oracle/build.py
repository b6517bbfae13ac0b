"""Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.

Recipe: g++ -O2 -std=c++17 -shared -fPIC -ffp-contract=off -pthread on
oracle.cpp only.  The reference project itself cannot be compiled here (its
Galois, cxxopts and spdlog submodules are empty and MPI/Boost/libnuma are
absent), so there is no oracle/_ref build.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "oracle.cpp"
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if OUT.exists() and not force and OUT.stat().st_mtime >= max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
        return OUT
    cxx = shutil.which("g++") or "g++"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall",
           str(src), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{res.stdout}\n{res.stderr}")
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
