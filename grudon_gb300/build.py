"""In-tree build of libgrudon_gpu.so for sm_103a (nvcc, no cmake).

Every translation unit compiles in parallel into grudon_gb300/_build/ and the
shared library links with the static CUDA runtime, so loading it needs only
the driver.  Re-running is incremental: objects newer than every source and
header are kept.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libgrudon_gpu.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall",
             "-Wno-unused-function"]

CU_SOURCES = ["abi.cu", "pr_pull.cu", "graph_run.cu", "noalloc.cu", "msssp.cu", "policy.cu", "verify.cu", "layout_dev.cu"]
CPP_SOURCES = ["graph_tools.cpp", "layout.cpp", "policy_io.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build grudon_gb300")
    return cand


def _deps_mtime() -> float:
    files = list(CSRC.glob("*")) + list(INCLUDE.glob("**/*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _compile(src: Path, obj: Path, nvcc: str, verbose: bool) -> None:
    if src.suffix == ".cu":
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    else:
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {src.name}\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr.strip():
        print(res.stderr, file=sys.stderr)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles (incrementally) and returns the path of libgrudon_gpu.so."""
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    newest = _deps_mtime()
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    jobs = []
    for name in CU_SOURCES + CPP_SOURCES:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < newest:
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda j: _compile(j[0], j[1], nvcc, verbose), jobs))
    objs = [str(BUILD / (n + ".o")) for n in CU_SOURCES + CPP_SOURCES]
    tmp = BUILD / "libgrudon_gpu.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    build_cli(verbose)
    return LIB


CLI = BUILD / "grudon"


def build_cli(verbose: bool = False) -> Path:
    """The flag-compatible driver over the C++ plugin API (links the .so)."""
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, *CXX_FLAGS, "-I", str(INCLUDE), str(CSRC / "cli.cpp"), "-o", str(CLI), f"-L{BUILD}", "-lgrudon_gpu",
           "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"cli build failed\n{res.stdout}\n{res.stderr}")
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
