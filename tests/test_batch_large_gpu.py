"""Batched path at the serving sizes (up to 2000 beads), its list-overflow
fallback, blow-up detection and preemption / resume, on the GPU."""
import numpy as np
import pytest

from conftest import rel_force_err

pytestmark = pytest.mark.gpu

# Per-term energy and trajectory tolerances of the parity tests.
E_TOL = 1e-5
X_TOL = 1e-5  # nm after 10 steps


def _spec(n, seed, T=300.0):
    from opencafemol_gb300 import synth
    return synth.go_protein(int(n), seed, temperature=float(T))


def _v0(n, seed):
    v = np.random.default_rng(seed).normal(scale=0.2, size=(n, 3))
    return v.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("n,T", [(1000, 285.0), (1500, 330.0), (2000, 355.0)])
def test_large_systems_match_oracle(gpu, n, T):
    """Forces, per-term energies and a 10-step trajectory of 1000-2000-bead
    Go proteins (the serving stream's sizes) against the FP64 oracle."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    s = _spec(n, 7000 + n, T)
    system = synth.build_system(s)
    b = gpu.Batch(max_systems=1, max_total_beads=2048, max_beads_per_system=2048)
    v0 = _v0(n, n)
    slot = b.admit(system, s.pos, velocities=v0, temperature=s.temperature, friction=s.friction,
                   step_size=s.dt, seed=21, n_steps=10)
    f, e = b.state(slot)
    f_ref, e_ref = oracle.evaluate(s)
    assert rel_force_err(f, f_ref) <= 1e-4
    for g, name in enumerate(system.group_names()):
        assert abs(e[g] - e_ref[name]) <= E_TOL * max(1.0, abs(e_ref[name])), name
    b.run(10, sync=True)
    x = s.pos.copy()
    v = v0.copy()
    oracle.simulate(s, x, v, 10, seed=21)
    assert np.max(np.abs(b.positions(slot) - x)) < X_TOL


def test_2000_bead_system_same_alone_and_in_mix(gpu):
    from opencafemol_gb300 import synth
    sizes = [2000, 64, 1200, 300, 1800, 90]
    temps = [340.0, 280.0, 300.0, 320.0, 290.0, 360.0]
    specs = [_spec(n, 7100 + k, T) for k, (n, T) in enumerate(zip(sizes, temps))]
    target = specs[0]
    sys_t = synth.build_system(target)
    alone = gpu.Batch(max_systems=1, max_total_beads=2048, max_beads_per_system=2048)
    a = alone.admit(sys_t, target.pos, temperature=target.temperature, seed=42, n_steps=200)
    for _ in range(2):
        alone.run(100)
    mix = gpu.Batch(max_systems=8, max_total_beads=sum(sizes) + 64, max_beads_per_system=2048)
    slots = [mix.admit(synth.build_system(s), s.pos, temperature=s.temperature, seed=7 + k, n_steps=200)
             for k, s in enumerate(specs[1:])]
    mix.retire(slots[1])  # a hole in the bead arena
    m = mix.admit(sys_t, target.pos, temperature=target.temperature, seed=42, n_steps=200)
    for _ in range(4):
        mix.run(50)
    assert np.array_equal(alone.positions(a), mix.positions(m))
    assert np.array_equal(alone.velocities(a), mix.velocities(m))


def _extended(n):
    """A straight chain with the protein's 0.38 nm bonds: few neighbours per
    bead, so the list capacity sized from it is far too small for the
    folded structure."""
    x = np.zeros((n, 3))
    x[:, 0] = 0.38 * np.arange(n)
    return x


def test_list_overflow_fallback_and_growth(gpu):
    """A system admitted extended and then given its folded positions
    overflows its neighbour list on the next launch: that launch runs on the
    direct scan, the list grows, and the trajectory is bit-identical to the
    same system admitted folded (no overflow at all); the forces of an
    overflowing evaluation match the oracle."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    s = _spec(600, 7200, 310.0)
    system = synth.build_system(s)
    v0 = _v0(s.n, 3)
    ext = _extended(s.n)
    # (a) overflow on the first launch, capacity grown afterwards
    a = gpu.Batch(max_systems=1, max_total_beads=1024, max_beads_per_system=1024)
    sa = a.admit(system, ext, temperature=s.temperature, seed=11, n_steps=120)
    cap0 = a.slot_stats(sa)["list_capacity"]
    a.set_positions_many([sa], s.pos, v0)
    a.run(60)
    a.run(60)
    assert a.slot_stats(sa)["list_capacity"] > cap0
    # (b) the same trajectory as without any overflow
    b = gpu.Batch(max_systems=1, max_total_beads=1024, max_beads_per_system=1024)
    sb = b.admit(system, s.pos, velocities=v0, temperature=s.temperature, seed=11, n_steps=120)
    cap_b = b.slot_stats(sb)["list_capacity"]
    b.run(120)
    assert cap_b > cap0
    assert np.array_equal(a.positions(sa), b.positions(sb))
    assert np.array_equal(a.velocities(sa), b.velocities(sb))
    # (c) an evaluation that overflows uses the scan: forces against the oracle
    c = gpu.Batch(max_systems=1, max_total_beads=1024, max_beads_per_system=1024)
    sc = c.admit(system, ext, temperature=s.temperature, seed=11, n_steps=1)
    c.set_positions_many([sc], s.pos)
    f, e = c.state(sc)
    f_ref, e_ref = oracle.evaluate(s)
    assert rel_force_err(f, f_ref) <= 1e-4
    for g, name in enumerate(system.group_names()):
        assert abs(e[g] - e_ref[name]) <= E_TOL * max(1.0, abs(e_ref[name])), name


def test_blown_up_system_is_reported_and_isolated(gpu):
    """Two beads of one system placed 0.01 nm apart (a finite input whose
    excluded-volume force is ~1e23 kJ/mol/nm): that slot stops after its
    first step and reports NONFINITE; the other systems of the launch run
    exactly as in a batch without it."""
    from opencafemol_gb300 import synth
    specs = [_spec(n, 7300 + k) for k, n in enumerate([120, 250, 80])]
    bad = specs[1].pos.copy()
    bad[200] = bad[10] + np.array([0.01, 0.0, 0.0])
    mixed = gpu.Batch(max_systems=3, max_total_beads=512, max_beads_per_system=512)
    slots = []
    for k, s in enumerate(specs):
        slots.append(mixed.admit(synth.build_system(s), bad if k == 1 else s.pos, seed=5 + k, n_steps=100))
    with pytest.raises(gpu.OCMError) as ei:
        mixed.state(slots[1])
    assert ei.value.code == 7
    mixed.run(50)
    mixed.run(50)
    assert mixed.status(slots[1]) == 7
    assert mixed.steps_done(slots[1]) == 1
    assert sorted(mixed.finished()) == sorted(slots)
    assert mixed.status(slots[0]) == 0 and mixed.status(slots[2]) == 0
    clean = gpu.Batch(max_systems=2, max_total_beads=512, max_beads_per_system=512)
    c0 = clean.admit(synth.build_system(specs[0]), specs[0].pos, seed=5, n_steps=100)
    c2 = clean.admit(synth.build_system(specs[2]), specs[2].pos, seed=7, n_steps=100)
    clean.run(100)
    assert np.array_equal(clean.positions(c0), mixed.positions(slots[0]))
    assert np.array_equal(clean.positions(c2), mixed.positions(slots[2]))


def test_preempt_and_resume(gpu):
    """A trajectory taken out of a batch after 40 of its 100 steps and
    admitted again (another batch, another slot) with its positions,
    velocities and step count ends exactly where the uninterrupted one does."""
    from opencafemol_gb300 import synth
    s = _spec(450, 7400, 295.0)
    system = synth.build_system(s)
    full = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
    sf = full.admit(system, s.pos, temperature=s.temperature, seed=99, n_steps=100)
    full.run(100)
    first = gpu.Batch(max_systems=2, max_total_beads=1024, max_beads_per_system=512)
    other = _spec(300, 7401)
    first.admit(synth.build_system(other), other.pos, seed=1, n_steps=10 ** 6)
    s1 = first.admit(system, s.pos, temperature=s.temperature, seed=99, n_steps=100)
    first.run(40)
    x, v, done = first.positions(s1), first.velocities(s1), first.steps_done(s1)
    first.retire(s1)
    assert done == 40
    second = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
    s2 = second.admit(system, x, velocities=v, temperature=s.temperature, seed=99, n_steps=100,
                      steps_done=done)
    second.run(25)
    second.run(50)
    assert second.steps_done(s2) == 100
    assert np.array_equal(second.positions(s2), full.positions(sf))
    assert np.array_equal(second.velocities(s2), full.velocities(sf))
