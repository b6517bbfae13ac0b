"""Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.

Recipe: g++ -O2 -std=c++17 -shared -fPIC -ffp-contract=off -pthread on
oracle.cpp (the restated round protocol and textbook oracles),
graphgen.cpp (the restated benchmark-graph generators) and pagerank.cpp (the
FP32-Kahan Jacobi PageRank of the PageRank workload).  The reference project itself cannot be compiled here (its
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
    srcs = [HERE / "oracle.cpp", HERE / "graphgen.cpp", HERE / "pagerank.cpp"]
    OUT.parent.mkdir(parents=True, exist_ok=True)
    newest = max([f.stat().st_mtime for f in srcs] + [Path(__file__).stat().st_mtime])
    if OUT.exists() and not force and OUT.stat().st_mtime >= newest:
        return OUT
    cxx = shutil.which("g++") or "g++"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall",
           *[str(f) for f in srcs], "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{res.stdout}\n{res.stderr}")
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
