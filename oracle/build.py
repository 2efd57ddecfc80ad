"""Build the FP64 CPU oracle (test infrastructure) into oracle/build/liboracle.so.

Plain g++; -ffp-contract=off so the FP32 cutoff emulation and the minimum
scans round exactly as written; OpenMP is not used (the CPU baseline runs
independent systems on separate threads from Python).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "ocm_oracle.cpp"
HDR = HERE / "oracle_tables.h"
OUT = HERE / "build" / "liboracle.so"


def build(verbose: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return OUT
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
           "-ffp-contract=off", "-Wall", str(SRC), "-o", str(OUT) + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(str(OUT) + ".tmp", OUT)
    if verbose:
        print(f"[build] {OUT}", file=sys.stderr)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
