"""Build the in-tree shared library ``opencafemol_gb300/lib/libocm_gb300.so``.

Every CUDA translation unit is compiled for sm_103a only; host C++ units are
compiled with ``-ffp-contract=off`` so the generators' parameter scans round
exactly as written on both x86-64 and aarch64.  Translation units are
compiled in parallel and skipped when their object is newer than every
source and header.
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
INCLUDE = PKG.parent / "include"
OBJ = PKG / "_build"
LIB = PKG / "lib" / "libocm_gb300.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + [
    "-O3", "-lineinfo", "-std=c++17",
    "--ftz=true", "--prec-div=false", "--prec-sqrt=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-I", str(INCLUDE),
]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
             "-I", str(CUDA_HOME / "include"), "-I", str(INCLUDE)]

CU_SOURCES = ["plain_engine.cu", "batch_engine.cu"]
CXX_SOURCES = ["host_system.cpp", "tables.cpp", "capi.cpp", "minimize.cpp"]


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + \
        sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(cmd: list[str], what: str) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {what} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if "-v" in cmd:  # ptxas resource report requested
        print(r.stderr, file=sys.stderr)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile (incrementally) and link the library; return its path."""
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError(f"nvcc not found at {NVCC}")
    OBJ.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    deps = _headers()
    jobs = []
    objs = []
    for name in CU_SOURCES:
        src, obj = CSRC / name, OBJ / (name + ".o")
        objs.append(obj)
        if _stale(obj, src, deps) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append(([NVCC, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)], name))
    for name in CXX_SOURCES:
        src, obj = CSRC / name, OBJ / (name + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append(([CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)], name))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        futs = {ex.submit(_compile, cmd, name): name for cmd, name in jobs}
        for f in cf.as_completed(futs):
            f.result()
            if verbose:
                print(f"[build] compiled {futs[f]}", file=sys.stderr)
    if jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [NVCC, *GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static",
               "-lrt", "-lpthread", "-ldl"]
        _compile(cmd, "link")
        os.replace(tmp, LIB)
        if verbose:
            print(f"[build] linked {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
