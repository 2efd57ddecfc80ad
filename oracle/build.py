"""Build the CPU test infrastructure into oracle/build/liboracle.so: the FP64
oracle (ocm_oracle.cpp) and the timed FP32 CPU restatement
(cpu_baseline.cpp).

Plain g++.  The oracle is compiled with -ffp-contract=off so the FP32 cutoff
emulation and the minimum scans round exactly as written; the CPU
restatement with -O3 and OpenMP (it runs an ensemble's systems on all host
cores).  Both objects are linked into one library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = {"ocm_oracle.cpp": ["-O2", "-ffp-contract=off"],
           "cpu_baseline.cpp": ["-O3", "-fopenmp"]}
HEADERS = [HERE / "oracle_tables.h", HERE / "oracle_system.h"]
OUT = HERE / "build" / "liboracle.so"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(map(str, cmd))}\n{r.stderr}")


def build(verbose: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    deps = [HERE / s for s in SOURCES] + HEADERS + [Path(__file__)]
    if OUT.exists() and OUT.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return OUT
    cxx = os.environ.get("CXX", "g++")
    objs = []
    cmds = []
    for src, flags in SOURCES.items():
        obj = OUT.parent / (Path(src).stem + ".o")
        objs.append(obj)
        cmds.append([cxx, *flags, "-std=c++17", "-fPIC", "-Wall", "-c", str(HERE / src), "-o", str(obj)])
    with ThreadPoolExecutor(len(cmds)) as ex:
        list(ex.map(_run, cmds))
    _run([cxx, "-shared", "-fopenmp", *map(str, objs), "-o", str(OUT) + ".tmp"])
    os.replace(str(OUT) + ".tmp", OUT)
    if verbose:
        print(f"[build] {OUT}", file=sys.stderr)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
