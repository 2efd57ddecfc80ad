"""Trajectory and energy files in the reference's formats
(src/Observer.cpp): DCD records, the .ene columns, and the run loop of
src/Simulator.cpp:50-76 with output written by a background thread."""
import struct

import numpy as np
import pytest


def test_dcd_roundtrip(tmp_path):
    from opencafemol_gb300 import observers as ob
    p = tmp_path / "t.dcd"
    x = np.random.default_rng(0).normal(size=(5, 3))
    with open(p, "wb") as fh:
        ob.write_dcd_header(fh, 5, total_frames=2, save_interval=10, total_step=20, delta_t=0.4,
                            use_periodic=True)
        ob.write_dcd_frame(fh, x, box_angstrom=(100.0, 120.0, 140.0))
        ob.write_dcd_frame(fh, x + 1, box_angstrom=(100.0, 120.0, 140.0))
    raw = p.read_bytes()
    assert struct.unpack_from("<i", raw, 0)[0] == 84 and raw[4:8] == b"CORD"
    d = ob.read_dcd(p)
    assert (d["total_frames"], d["save_interval"], d["total_step"], d["version"]) == (2, 10, 20, 24)
    assert d["delta_t"] == pytest.approx(0.4) and d["has_unitcell"] and d["n_particles"] == 5
    assert np.array_equal(d["frames"][0], x.astype(np.float32))
    assert np.array_equal(d["frames"][1], (x + 1).astype(np.float32))
    assert d["unitcells"][0].tolist() == [100.0, 90.0, 120.0, 90.0, 90.0, 140.0]


def test_energy_file_layout():
    from opencafemol_gb300 import observers as ob

    class FakeSystem:
        def group_names(self):
            return ["HarmonicBond", "GoContact", "ExcludedVolume"]

    e = ob.EnergyObserver("x", FakeSystem())
    head = e.header().splitlines()
    assert head[0] == "# unit of energy : kcal/mol"
    # name order, as the reference's std::map<name, group>
    assert head[1] == "# timestep" + f" {'ExcludedVolume':>24}" + f" {'GoContact':>24}" + \
        f" {'HarmonicBond':>24}" + " kinetic_energy"
    line = e.line(100, np.array([4.184, -8.368, 41.84]), 12.552)
    assert line == f"{100:<10d}" + f" {10.0:>24.6f}" + f" {-2.0:>24.6f}" + f" {1.0:>24.6f}" + \
        f" {3.0:>14.6f}\n"


@pytest.mark.gpu
def test_simulator_writes_frames(gpu, tmp_path):
    from opencafemol_gb300 import observers as ob
    from opencafemol_gb300 import synth
    spec = synth.go_protein(60, 71)
    system = synth.build_system(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(spec.pos)
    ctx.setVelocitiesToTemperature(300.0, 3)
    prefix = tmp_path / "run"
    sim = ob.Simulator(ctx, total_step=30, save_step=10, observers=[
        ob.EnergyObserver(prefix, system), ob.DCDObserver(prefix, 30, 10, 0.2, False),
        ob.PDBObserver(prefix, ["ALA"] * spec.n)])
    sim.run()
    assert ctx.stats()["steps_done"] == 30
    d = ob.read_dcd(str(prefix) + "_position.dcd")
    assert d["frames"].shape == (3, spec.n, 3) and d["total_frames"] == 3
    assert np.allclose(d["frames"][0], spec.pos * 10.0, atol=1e-4)
    v = ob.read_dcd(str(prefix) + "_velocity.dcd")
    assert v["frames"].shape == (3, spec.n, 3)
    ene = (tmp_path / "run.ene").read_text().splitlines()
    assert len(ene) == 2 + 3 and ene[2].startswith("0 ") and ene[4].startswith("20 ")
    assert (tmp_path / "run.pdb").read_text().count("ENDMDL") == 3
