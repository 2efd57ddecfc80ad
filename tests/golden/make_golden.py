"""Generate the golden fixtures under tests/golden/ from the reference's own
sample inputs.

The reference ships no expected outputs (its tests only check that inputs
parse), so the expected values here are the FP64 oracle's, evaluated on
systems read from the reference's sample TOML files:

* ``sh3_aicg2.npz``: sample/toml_input/sh3_AICG2+.toml, all 56 beads and
  every term of the file: HarmonicBond, GoContact, GaussianBond,
  FlexibleLocalAngle, GaussianDihedral, FlexibleLocalDihedral and
  ExcludedVolume;
* ``fus_hps_2chains.npz``: the first two 163-bead chains of
  sample/toml_input/FUS_100_HPS.toml in the file's periodic box, with
  HarmonicBond, LennardJonesRepulsive, LennardJonesAttractive and
  DebyeHuckel.

Each fixture holds the full input description (so tests rebuild the system
without the TOML file) and the oracle forces and per-term energies.  The
sh3 fixture (a native structure) also holds a 10-step Langevin trajectory
of the oracle.  The FUS excerpt is an unminimised start (the reference runs
an energy minimisation before dynamics; beads overlap at 0.21 nm with sigma
up to 0.75 nm, forces up to ~7e7 kJ/mol/nm), so it pins forces and energies
at a large-force configuration and carries no trajectory.

    python tests/golden/make_golden.py [path/to/sample/toml_input]
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from opencafemol_gb300 import synth, toml_input  # noqa: E402
from oracle import oracle  # noqa: E402

TRAJ_STEPS = 10
TRAJ_SEED = 2024
CASES = {  # name: (file, beads kept (None = all), dt (ps), with trajectory)
    "sh3_aicg2": ("sh3_AICG2+.toml", None, 0.01, True),
    "fus_hps_2chains": ("FUS_100_HPS.toml", 326, 0.01, False),
}


def make(sample_dir: Path) -> dict:
    manifest = {}
    for name, (fname, n_keep, dt, traj) in CASES.items():
        path = sample_dir / fname
        raw = path.read_bytes()
        t = toml_input.read_toml(raw, strict=False)
        spec = t.spec if n_keep is None else synth.subset_spec(t.spec, n_keep)
        # a 10 fs step (the benchmark's), not the sample's own delta_t
        spec.dt = dt
        forces, energies = oracle.evaluate(spec)
        arrays = synth.spec_to_arrays(spec)
        arrays.update(forces=forces, energy_names=np.array(list(energies)),
                      energies=np.array(list(energies.values())))
        if traj:
            x = spec.pos.copy()
            v = np.zeros_like(x)
            oracle.simulate(spec, x, v, TRAJ_STEPS, seed=TRAJ_SEED)
            arrays.update(traj_pos=x, traj_vel=v, traj_meta=np.array([TRAJ_STEPS, TRAJ_SEED]))
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        manifest[name] = {"source": f"sample/toml_input/{fname}",
                          "source_sha256": hashlib.sha256(raw).hexdigest(),
                          "beads": int(spec.n), "skipped_terms": t.skipped,
                          "energies_kj_mol": {k: float(v_) for k, v_ in energies.items() if v_ != 0.0},
                          "max_force_kj_mol_nm": float(np.linalg.norm(forces, axis=1).max()),
                          "trajectory": {"steps": TRAJ_STEPS, "seed": TRAJ_SEED, "dt_ps": dt,
                                         "initial_velocity": "zero"} if traj else None}
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")
    return manifest


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference>/sample/toml_input")
    print(json.dumps(make(Path(sys.argv[1])), indent=1))
