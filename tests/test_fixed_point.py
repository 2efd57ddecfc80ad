"""The integer-only read-out of the 64-bit fixed-point force accumulators
agrees with IEEE-754 round-half-even (host build of the same header the
kernels include)."""
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_fixed_point_conversions(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "fixed_point_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", str(ROOT / "opencafemol_gb300" / "csrc"),
                    str(ROOT / "tests" / "fixed_point_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "1500000"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 mismatches" in out.stdout
