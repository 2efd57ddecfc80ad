"""Device-side detection of a blown-up system on the plain path: a finite
input whose forces exceed what the engine can represent (two beads 0.01 nm
apart: excluded-volume force ~1e23 kJ/mol/nm) is reported as NONFINITE by
getState and step; step leaves the context in its state from before the
call.  The failure is made on the host (positions); no GPU fault is
involved."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _overlapping(n=120, seed=35):
    from opencafemol_gb300 import synth
    spec = synth.go_protein(n, seed)
    x = spec.pos.copy()
    x[100] = x[10] + np.array([0.01, 0.0, 0.0])
    return spec, x


def test_plain_get_state_reports_blow_up(gpu):
    from opencafemol_gb300 import synth
    spec, x = _overlapping()
    ctx = gpu.Context(synth.build_system(spec), gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(x)
    with pytest.raises(gpu.OCMError) as ei:
        ctx.getState()
    assert ei.value.code == 7
    # the same context evaluates normally once the overlap is gone
    ctx.setPositions(spec.pos)
    f, e = ctx.getState()
    assert np.all(np.isfinite(f)) and np.isfinite(e)


@pytest.mark.parametrize("engine", ["tiles", "one_system"])
def test_plain_step_reports_blow_up_and_keeps_state(gpu, engine):
    from opencafemol_gb300 import synth
    spec, x = _overlapping()
    ctx = gpu.Context(synth.build_system(spec), gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3), engine=engine)
    ctx.setPositions(x)
    ctx.setVelocitiesToTemperature(300.0, 4)
    v0 = ctx.getVelocities()
    with pytest.raises(gpu.OCMError) as ei:
        ctx.step(10)
    assert ei.value.code == 7
    assert np.array_equal(ctx.getPositions(), x)
    assert np.array_equal(ctx.getVelocities(), v0)
    assert ctx.stats()["steps_done"] == 0


def test_periodic_blow_up_is_reported(gpu):
    """The same check on a periodic HPS slab (tiles and charged rows)."""
    from opencafemol_gb300 import synth
    spec = synth.hps_slab(20, 50, (10.0, 10.0, 40.0), slab_width=10.0, seed=8)
    x = spec.pos.copy()
    x[500] = x[3] + np.array([0.005, 0.0, 0.0])
    ctx = gpu.Context(synth.build_system(spec), gpu.LangevinIntegrator(300.0, 0.1, 0.01, 3))
    ctx.setPositions(x)
    with pytest.raises(gpu.OCMError) as ei:
        ctx.step(5)
    assert ei.value.code == 7
