"""Host-side pieces of the benchmark: the roofline arithmetic and the
reference arm's JSON line (the CPU restatement, runnable without a GPU)."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT


def test_roofline_object_is_json():
    import bench
    specs = bench.ensemble_specs(count=6)
    roof = bench.batched_roofline(specs, K=10, launch_s=1e-3, sm_max_mhz=2070.0, traffic=None, sms=152)
    json.dumps(roof)
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    beads = sum(s.n for s in specs)
    # 16 + 24 + 100 B per bead plus 4 B per pair and the bonded records
    assert roof["bytes_per_bead_step"] > 140
    assert roof["algorithmic_bytes_per_launch"] == pytest.approx(roof["bytes_per_bead_step"] * beads * 10)
    assert 0 < roof["frac"] and 0 < roof["fp32"]["frac"]


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--md-steps", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["value"] > 0
    # the whole 512-replica workload, and the engine library never mapped
    assert line["config"]["replicas"] == 512 and line["config"]["md_steps_per_step"] == 2
    assert line["engine_library_loaded"] is False


def test_clock_records_that_force_a_remeasure():
    import bench
    ok = {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []}
    assert not bench.clocks_rejected(ok)
    assert not bench.clocks_rejected(dict(ok, sm_mhz=1800.0, reasons=["sw_power_cap"]))  # kept, noted
    for r in ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"):
        assert bench.clocks_rejected(dict(ok, reasons=[r]))
    assert bench.clocks_rejected(dict(ok, sm_mhz=1400.0))  # well below max, no reason: a clock lock
    assert not bench.clocks_rejected(dict(ok, sm_mhz=1950.0))
    assert not bench.clocks_rejected({"reasons": [], "samples": 0})  # no samples: nothing to judge
