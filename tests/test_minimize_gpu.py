"""Local energy minimisation (the reference's optional step before a run,
src/Simulator.cpp:41-46) on the plain context: L-BFGS until the RMS of all
force components is at most the tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rms(f):
    return float(np.sqrt(np.mean(f * f)))


@pytest.mark.parametrize("kind", ["go", "slab"])
def test_minimize_reaches_tolerance(gpu, kind):
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = (synth.go_protein(200, 31) if kind == "go"
            else synth.hps_slab(30, 100, (15.0, 15.0, 60.0), slab_width=20.0, seed=9))
    system = synth.build_system(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(spec.pos)
    f0, e0 = ctx.getState()
    tol = 10.0
    it = gpu.LocalEnergyMinimizer.minimize(ctx, tol)
    f1, e1 = ctx.getState()
    assert it > 0 and e1 < e0
    assert _rms(f1) <= tol < _rms(f0)
    # the minimised structure is a minimum for the FP64 oracle too
    x = ctx.getPositions()
    f_ref, _ = oracle.evaluate(spec, pos=x)
    assert _rms(f_ref) <= 1.01 * tol


def test_minimize_iteration_limit_and_simulator(gpu, tmp_path):
    from opencafemol_gb300 import observers, synth
    spec = synth.go_protein(120, 32)
    system = synth.build_system(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(spec.pos)
    _, e0 = ctx.getState()
    assert gpu.LocalEnergyMinimizer.minimize(ctx, 1e-6, 5) == 5
    _, e1 = ctx.getState()
    assert e1 < e0
    with pytest.raises(gpu.OCMError):
        gpu.LocalEnergyMinimizer.minimize(ctx, -1.0)
    sim = observers.Simulator(ctx, 20, 10, [observers.EnergyObserver(tmp_path / "m", system)],
                              energy_minimization=True)
    sim.initialize(spec.pos)
    f, _ = ctx.getState()
    assert _rms(f) <= 10.0
    sim.run()
    assert (tmp_path / "m.ene").exists()


def test_minimize_reports_why_it_stopped(gpu):
    """The stop reason and the final RMS force are reported: converged at a
    reachable tolerance, the iteration limit, and a tolerance below the FP32
    force floor ends as stagnation (or a failed line search), not a hang."""
    from opencafemol_gb300 import synth
    spec = synth.go_protein(150, 33)
    system = synth.build_system(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(spec.pos)
    with pytest.raises(gpu.OCMError) as ei:
        gpu.LocalEnergyMinimizer.report(ctx)
    assert ei.value.code == 5
    gpu.LocalEnergyMinimizer.minimize(ctx, 10.0)
    r = gpu.LocalEnergyMinimizer.report(ctx)
    assert r["code"] == 0 and r["rms_force"] <= 10.0
    ctx.setPositions(spec.pos)
    gpu.LocalEnergyMinimizer.minimize(ctx, 1e-9, 3)
    assert gpu.LocalEnergyMinimizer.report(ctx)["code"] == 1
    ctx.setPositions(spec.pos)
    gpu.LocalEnergyMinimizer.minimize(ctx, 1e-9)
    r = gpu.LocalEnergyMinimizer.report(ctx)
    assert r["code"] in (2, 3) and r["rms_force"] > 1e-9


def test_minimize_from_overlap_and_blown_start(gpu):
    """An overlap of 0.2 nm (forces ~1e7 kJ/mol/nm) is minimised; a start
    with two beads 0.01 nm apart (forces ~1e23) is refused as NONFINITE."""
    from opencafemol_gb300 import synth
    spec = synth.go_protein(120, 34)
    system = synth.build_system(spec)
    x = spec.pos.copy()
    x[100] = x[10] + np.array([0.2, 0.0, 0.0])
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(x)
    gpu.LocalEnergyMinimizer.minimize(ctx, 10.0)
    f, _ = ctx.getState()
    assert _rms(f) <= 10.0
    x[100] = x[10] + np.array([0.01, 0.0, 0.0])
    ctx.setPositions(x)
    with pytest.raises(gpu.OCMError) as ei:
        gpu.LocalEnergyMinimizer.minimize(ctx, 10.0)
    assert ei.value.code == 7
