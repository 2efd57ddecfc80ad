"""Precision study of the plain path on an HPS condensate slab (FP32 pair
arithmetic, 64-bit fixed-point forces, FP64 energy sums, FP64 kinetic
reduction, FP64 master positions) against the FP64 oracle:

* per-bead force error and per-term energy error at a relaxed configuration
  (the oracle enumerates pairs on a cell grid);
* the kinetic energy reduction against an FP64 sum of the same velocities;
* total-energy drift of an NVE run (gamma = 0, dt = 5 fs, 10^4 steps).

Size: OCM_PRECISION_CHAINS chains of 200 beads (default 1000, i.e. 200,000
beads in a 30 x 30 x 300 nm box, the precision configuration; 100 or fewer
chains use a 15 x 15 x 150 nm box).  The energy drift is asserted against
a stated bound.
The measured numbers are printed as one JSON line (and written to the file
named by OCM_PRECISION_REPORT, if set)."""
import json
import os

import numpy as np
import pytest

from conftest import rel_force_err, rms_rel_err

pytestmark = pytest.mark.gpu

BOLTZ = 0.00831446261815324
# |NVE drift| bound, kT per bead per ns, at dt = 5 fs (FP32 pair arithmetic
# with FP64 master positions and fixed-point forces)
DRIFT_BOUND = 1e-2


def _slab():
    from opencafemol_gb300 import synth
    chains = int(os.environ.get("OCM_PRECISION_CHAINS", "1000"))
    if chains <= 100:
        box, width = (15.0, 15.0, 150.0), 30.0
    else:
        box, width = (30.0, 30.0, 300.0), 60.0
    return synth.hps_slab(chains, 200, box, slab_width=width, seed=31)


def test_precision_study(gpu):
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = _slab()
    system = synth.build_system(spec)
    # relax the random packing (strong friction, 2 fs), then take the
    # configuration in the box frame, FP32-exact, as the common input
    rel = gpu.Context(system, gpu.LangevinIntegrator(300.0, 5.0, 0.002, 3))
    rel.setPositions(spec.pos)
    rel.setVelocitiesToTemperature(300.0, 3)
    rel.step(3000)
    L = np.array(spec.box)
    x = rel.getPositions()
    x = x - L * np.floor(x / L)
    x = x.astype(np.float32).astype(np.float64)
    x = np.where(x >= L, x - L, x)
    del rel

    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.0, 0.005, 9))
    ctx.setPositions(x)
    f, etot = ctx.getState()
    e32 = ctx.getGroupEnergies()
    got = {nm: e32[g] for g, nm in enumerate(system.group_names())}
    f_ref, e_ref = oracle.evaluate(spec, pos=x, cells=1)
    force_max = rel_force_err(f, f_ref)
    force_rms = rms_rel_err(f, f_ref)
    e_err = {k: abs(got[k] - v) / max(1.0, abs(v)) for k, v in e_ref.items() if v != 0.0}

    # kinetic energy: device FP64 reduction vs an FP64 sum of the same FP32
    # velocities and the same FP32 inverse masses (the reduction's error),
    # and vs the FP64 masses (adds the FP32 rounding of 1/m)
    ctx.setVelocitiesToTemperature(300.0, 17)
    v = ctx.getVelocities()
    invm32 = (1.0 / spec.masses).astype(np.float32).astype(np.float64)
    ke_dev = ctx.getKineticEnergy()
    ke_host = 0.5 * float(np.sum(v * v / invm32[:, None]))
    ke_err = abs(ke_dev - ke_host) / ke_host
    ke_host64 = 0.5 * float(np.sum(spec.masses[:, None] * v * v))
    ke_err_mass = abs(ke_dev - ke_host64) / ke_host64

    # NVE drift: total energy every 500 steps over 10^4 steps of 5 fs
    energies = []
    for _ in range(21):
        _, pe = ctx.getState(forces=False)
        energies.append(pe + ctx.getKineticEnergy())
        ctx.step(500)
    energies = np.array(energies)
    t_ps = np.arange(len(energies)) * 500 * 0.005
    slope = float(np.polyfit(t_ps, energies, 1)[0])  # kJ/mol/ps
    kT = BOLTZ * 300.0
    drift = slope / (spec.n * kT) * 1000.0  # kT per bead per ns
    fluct = float(np.std(energies - np.polyval(np.polyfit(t_ps, energies, 1), t_ps)))

    report = {"beads": int(spec.n), "box_nm": list(spec.box), "force_max_rel": force_max,
              "force_rms_rel": force_rms, "energy_rel": e_err, "kinetic_rel": ke_err,
              "kinetic_rel_fp64_masses": ke_err_mass,
              "nve_steps": 10000, "nve_dt_ps": 0.005, "nve_drift_kT_per_bead_per_ns": drift,
              "nve_fluct_kj_mol": fluct, "nve_E0_kj_mol": float(energies[0])}
    line = json.dumps(report)
    print(line)
    out = os.environ.get("OCM_PRECISION_REPORT")
    if out:
        with open(out, "w") as fh:
            fh.write(line + "\n")
    assert force_max <= 1e-4
    assert force_rms <= 1e-5
    assert max(e_err.values()) <= 1e-5
    assert ke_err <= 1e-12
    assert np.all(np.isfinite(energies))
    assert abs(drift) <= DRIFT_BOUND
