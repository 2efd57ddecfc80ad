"""Batched / served path on the GPU: parity with the FP64 oracle, identical
results alone and in a mix, continuous admission and retirement."""
import numpy as np
import pytest

from conftest import rel_force_err

pytestmark = pytest.mark.gpu


def _systems(sizes, seed0=100, temps=None):
    from opencafemol_gb300 import synth
    specs = []
    for k, n in enumerate(sizes):
        T = 300.0 if temps is None else float(temps[k])
        specs.append(synth.go_protein(int(n), seed0 + k, temperature=T))
    return specs


def test_batch_forces_match_oracle(gpu):
    from opencafemol_gb300 import synth
    from oracle import oracle
    specs = _systems([50, 97, 256, 333, 800], temps=[280, 300, 320, 340, 360])
    batch = gpu.Batch(max_systems=8, max_total_beads=4096, max_beads_per_system=800)
    slots = []
    for s in specs:
        system = synth.build_system(s)
        slots.append((batch.admit(system, s.pos, temperature=s.temperature, n_steps=10), system, s))
    for slot, system, s in slots:
        f, e32 = batch.state(slot)
        f_ref, e_ref = oracle.evaluate(s)
        assert rel_force_err(f, f_ref) <= 1e-4
        names = system.group_names()
        for g, name in enumerate(names):
            assert abs(e32[g] - e_ref[name]) <= 1e-5 * max(1.0, abs(e_ref[name])), name


def test_same_alone_and_in_mix(gpu):
    """A system's trajectory does not depend on what else is in the batch."""
    from opencafemol_gb300 import synth
    specs = _systems([64, 300, 150, 700, 90], seed0=200)
    target = specs[1]
    sys_t = synth.build_system(target)
    alone = gpu.Batch(max_systems=2, max_total_beads=1024, max_beads_per_system=800)
    a = alone.admit(sys_t, target.pos, seed=42, n_steps=300)
    for _ in range(3):
        alone.run(100)
    xa = alone.positions(a)

    mix = gpu.Batch(max_systems=8, max_total_beads=4096, max_beads_per_system=800)
    slots = [mix.admit(synth.build_system(s), s.pos, seed=7 + k, n_steps=300) for k, s in enumerate(specs)]
    mix.retire(slots[0])  # leave a hole in the bead arena
    m = mix.admit(sys_t, target.pos, seed=42, n_steps=300)
    for _ in range(3):
        mix.run(100)
    xm = mix.positions(m)
    assert np.array_equal(xa, xm)


def test_threads_per_cta_do_not_change_results(gpu):
    """The launch shape is a tuning knob only: 256, 512 and 1024 threads per
    CTA give bit-identical trajectories (small systems split their pair
    lists over lanes by a rule that depends on the bead count alone)."""
    from opencafemol_gb300 import synth
    specs = _systems([40, 100, 250, 600], seed0=900)
    out = []
    for th in (512, 256, 1024):
        b = gpu.Batch(max_systems=4, max_total_beads=2048, max_beads_per_system=800)
        b.set_threads(th)
        slots = [b.admit(synth.build_system(s), s.pos, seed=3 + k, n_steps=150) for k, s in enumerate(specs)]
        b.run(150)
        out.append([b.positions(k) for k in slots])
    for other in out[1:]:
        for xa, xb in zip(out[0], other):
            assert np.array_equal(xa, xb)


def test_chunking_does_not_change_results(gpu):
    from opencafemol_gb300 import synth
    s = _systems([400], seed0=300)[0]
    system = synth.build_system(s)
    out = []
    for chunks in ([240], [100, 100, 40], [7] * 34 + [2]):
        b = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
        slot = b.admit(system, s.pos, seed=9, n_steps=240)
        for c in chunks:
            b.run(c)
        assert b.steps_done(slot) == 240
        out.append(b.positions(slot))
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])


def test_batch_matches_plain_after_one_step(gpu):
    """The batched and the plain engine evaluate the same physics: after one
    step from identical state they agree to FP32 accumulation error."""
    from opencafemol_gb300 import synth
    s = _systems([256], seed0=400)[0]
    system = synth.build_system(s)
    v0 = np.random.default_rng(1).normal(scale=0.1, size=(s.n, 3)).astype(np.float32).astype(np.float64)
    b = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
    slot = b.admit(system, s.pos, velocities=v0, temperature=s.temperature, seed=77, n_steps=1)
    b.run(1)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(s.temperature, s.friction, s.dt, 77), engine="tiles")
    ctx.setPositions(s.pos)
    ctx.setVelocities(v0)
    ctx.step(1)
    assert np.max(np.abs(b.positions(slot) - ctx.getPositions())) < 1e-7
    assert np.max(np.abs(b.velocities(slot) - ctx.getVelocities())) < 1e-4


def test_continuous_admission(gpu):
    """Requests admitted while others run; finished ones retire and free
    capacity for new ones; every request completes its step count."""
    from opencafemol_gb300 import synth
    specs = _systems([40, 120, 500, 60, 250, 80, 700, 33], seed0=500)
    steps = [30, 200, 120, 50, 90, 10, 150, 70]
    batch = gpu.Batch(max_systems=3, max_total_beads=1300, max_beads_per_system=800)
    pending = list(range(len(specs)))
    running = {}
    done = {}
    rounds = 0
    while pending or running:
        while pending:
            k = pending[0]
            try:
                slot = batch.admit(synth.build_system(specs[k]), specs[k].pos, seed=k, n_steps=steps[k])
            except gpu.OCMError as e:
                assert e.code == 3  # out of capacity: wait for a retirement
                break
            running[slot] = k
            pending.pop(0)
        batch.run(25)
        for slot in batch.finished():
            k = running.pop(slot)
            assert batch.steps_done(slot) == steps[k]
            done[k] = batch.positions(slot)
            batch.retire(slot)
        rounds += 1
        assert rounds < 200
    assert sorted(done) == list(range(len(specs)))
    assert all(np.all(np.isfinite(x)) for x in done.values())


def test_oversize_system_rejected(gpu):
    from opencafemol_gb300 import synth
    s = _systems([300], seed0=600)[0]
    b = gpu.Batch(max_systems=2, max_total_beads=1024, max_beads_per_system=256)
    with pytest.raises(gpu.OCMError) as ei:
        b.admit(synth.build_system(s), s.pos, n_steps=1)
    assert ei.value.code == 3


def test_autotune_keeps_results(gpu):
    """The autotuner times real launches under each launch shape and keeps
    the fastest; the trajectory equals an untuned run of the same steps."""
    from opencafemol_gb300 import synth
    specs = _systems([60, 333, 777], seed0=950)
    runs = []
    for tune in (True, False):
        b = gpu.Batch(max_systems=3, max_total_beads=1300, max_beads_per_system=800)
        slots = [b.admit(synth.build_system(s), s.pos, seed=5 + k, n_steps=10 ** 6) for k, s in enumerate(specs)]
        cands = ((512, 96), (1024, -1, 512), (256, 48, 128))
        if tune:
            res = b.autotune(steps_per_trial=20, candidates=cands)
            picked = (res["threads"], res["list_smem_kib"], res["split_beads"])
            assert picked in [c if len(c) == 3 else c + (0,) for c in cands] and len(res["trials"]) == 3
            assert b.threads() == res["threads"]
        else:
            b.run(2 * 2 * 20 * len(cands), sync=True)
        runs.append([b.positions(k) for k in slots])
    for xa, xb in zip(*runs):
        assert np.array_equal(xa, xb)


def test_aicg_gaussian_terms_both_engines(gpu):
    """AICG2+ Gaussian bonds and dihedrals (on a perturbed structure, so the
    wells exert force) in the batched and the plain engine against the oracle."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.add_aicg_gaussians(synth.go_protein(300, 960), seed=961)
    x = spec.pos + np.random.default_rng(5).normal(scale=0.02, size=spec.pos.shape)
    x = x.astype(np.float32).astype(np.float64)
    system = synth.build_system(spec)
    f_ref, e_ref = oracle.evaluate(spec, pos=x)
    b = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
    slot = b.admit(system, x, seed=1, n_steps=1)
    f, e32 = b.state(slot)
    assert rel_force_err(f, f_ref) <= 1e-4
    names = system.group_names()
    for g, name in enumerate(names):
        assert abs(e32[g] - e_ref[name]) <= 1e-5 * max(1.0, abs(e_ref[name])), name
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 1))
    ctx.setPositions(x)
    fp, _ = ctx.getState()
    assert rel_force_err(fp, f_ref) <= 1e-4
    ep = ctx.getGroupEnergies()
    for g, name in enumerate(names):
        assert abs(ep[g] - e_ref[name]) <= 1e-5 * max(1.0, abs(e_ref[name])), name


def test_cta_split_keeps_results(gpu):
    """With more resident systems than two per CTA, CTAs split into two
    groups of half their threads for the small systems; every trajectory is
    identical to the one advanced by whole CTAs."""
    from opencafemol_gb300 import synth
    rng = np.random.default_rng(77)
    sizes = [int(n) for n in rng.integers(30, 420, 340)]
    specs = [synth.go_protein(n, 3000 + k) for k, n in enumerate(sizes)]
    systems = [synth.build_system(s) for s in specs]
    runs = []
    for threads, split in ((512, 0), (512, 384), (1024, 512), (256, 128)):
        b = gpu.Batch(max_systems=len(specs), max_total_beads=sum(sizes) + 64, max_beads_per_system=512)
        slots = [b.admit(so, s.pos, seed=40 + k, n_steps=10 ** 6) for k, (so, s) in enumerate(zip(systems, specs))]
        b.set_threads(threads)
        b.set_split(split)
        b.run(30, sync=True)
        b.run(30, sync=True)
        runs.append(b.get_positions_many(slots))
    for r in runs[1:]:
        assert np.array_equal(r, runs[0])


def test_positions_reset_mid_run(gpu):
    """A batch whose positions are reset mid-run (far from where its lists
    were built) continues exactly as a fresh batch resumed from that state
    (same step counter, velocities)."""
    from opencafemol_gb300 import synth
    specs = _systems([90, 260, 540], seed0=970)
    systems = [synth.build_system(s) for s in specs]
    a = gpu.Batch(max_systems=3, max_total_beads=1024, max_beads_per_system=800)
    slots = [a.admit(so, s.pos, seed=30 + k, n_steps=10 ** 6) for k, (so, s) in enumerate(zip(systems, specs))]
    for _ in range(3):
        a.run(20, sync=True)
    v = [a.velocities(k) for k in slots]
    # back to the starting structures (far from where the lists were built)
    a.set_positions_many(slots, np.concatenate([s.pos for s in specs]))
    a.run(25, sync=True)
    a.run(25, sync=True)
    b = gpu.Batch(max_systems=3, max_total_beads=1024, max_beads_per_system=800)
    sb = [b.admit(so, s.pos, velocities=v[k], seed=30 + k, n_steps=10 ** 6, steps_done=60)
          for k, (so, s) in enumerate(zip(systems, specs))]
    b.run(50, sync=True)
    for ka, kb in zip(slots, sb):
        assert np.array_equal(a.positions(ka), b.positions(kb))
        assert np.array_equal(a.velocities(ka), b.velocities(kb))


def _lj_protein(n, seed):
    """A Go-model chain whose excluded volume is replaced by HPS-style
    Lennard-Jones repulsion and attraction (per-bead sigma and lambda), with
    its Debye-Hueckel charges: the general pair kernel."""
    from opencafemol_gb300 import synth
    s = synth.go_protein(n, seed)
    rng = np.random.default_rng(seed)
    sig = rng.uniform(0.3, 0.5, n)
    lam = rng.uniform(0.0, 1.0, n)
    ratio = 2.0 / (0.5 * (np.sort(sig)[-1] + np.sort(sig)[-2]))
    s.exv = None
    s.ljr = synth.PairTerm(ratio=ratio, p0=np.full(n, 0.2 * synth.KJ_PER_KCAL), p1=sig, ign_bond=3)
    s.lja = synth.PairTerm(ratio=ratio, p0=0.2 * lam * synth.KJ_PER_KCAL, p1=sig, ign_bond=3)
    return s


def test_cta_split_general_pair_kernel(gpu):
    """Small chains on the general pair kernel (Lennard-Jones terms): one
    chain's forces against the oracle, and every trajectory identical with
    and without the CTA split (more than two systems per CTA)."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    rng = np.random.default_rng(91)
    lengths = [int(n) for n in rng.integers(30, 300, 320)]
    specs = [_lj_protein(n, 4000 + k) for k, n in enumerate(lengths)]
    systems = [synth.build_system(s) for s in specs]
    one = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
    slot = one.admit(systems[0], specs[0].pos, seed=1, n_steps=1)
    f, _ = one.state(slot)
    f_ref, _ = oracle.evaluate(specs[0])
    assert rel_force_err(f, f_ref) <= 1e-4
    runs = []
    for threads, split in ((512, 0), (512, 384), (1024, 512)):
        b = gpu.Batch(max_systems=len(specs), max_total_beads=sum(lengths) + 64, max_beads_per_system=512)
        slots = [b.admit(so, s.pos, seed=50 + k, n_steps=10 ** 6) for k, (so, s) in enumerate(zip(systems, specs))]
        b.set_threads(threads)
        b.set_split(split)
        b.run(30, sync=True)
        b.run(30, sync=True)
        runs.append(b.get_positions_many(slots))
    for r in runs[1:]:
        assert np.array_equal(r, runs[0])


def test_many_slot_upload_rejects_non_finite(gpu):
    """A non-finite position in a many-slot upload is refused with
    OCM_ERR_NONFINITE and changes no slot's state."""
    from opencafemol_gb300 import synth
    specs = _systems([40, 130], seed0=990)
    b = gpu.Batch(max_systems=2, max_total_beads=256, max_beads_per_system=200)
    slots = [b.admit(synth.build_system(s), s.pos, n_steps=10) for s in specs]
    before = b.get_positions_many(slots)
    for bad in (np.nan, np.inf, -np.inf):
        xyz = before + 0.5
        xyz[150, 1] = bad
        with pytest.raises(gpu.OCMError) as ei:
            b.set_positions_many(slots, xyz, np.zeros_like(xyz))
        assert ei.value.code == 7
        assert np.array_equal(b.get_positions_many(slots), before)
    b.set_positions_many(slots, before + 0.5)
    assert np.array_equal(b.get_positions_many(slots), before + 0.5)
    with pytest.raises(ValueError):  # fewer values than the slots' beads
        b.set_positions_many(slots, before[:-1])
