"""Plain single-system path on the GPU against the FP64 oracle.

Tolerances: per-bead force error max_i |dF_i| / max(|F_i|, 1e-3 F_rms)
<= 1e-4 (FP32 pair arithmetic, 64-bit fixed-point accumulation); per-term
energies within 1e-5 relative (or 1e-5 kJ/mol absolute for near-zero sums).
"""
import numpy as np
import pytest

from conftest import rel_force_err, rms_rel_err

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-4
ENERGY_TOL = 1e-5


def _ctx(ocm, spec, seed=7, engine="tiles"):
    from opencafemol_gb300 import synth
    system = synth.build_system(spec)
    ctx = ocm.Context(system, ocm.LangevinIntegrator(spec.temperature, spec.friction, spec.dt, seed),
                      engine=engine)
    ctx.setPositions(spec.pos)
    return system, ctx


def _group_energy_map(system, e32):
    return {name: e32[g] for g, name in enumerate(system.group_names())}


def _check_energies(e_ref, got):
    for name, ref in e_ref.items():
        if name not in got:
            assert abs(ref) < 1e-12, name
            continue
        tol = ENERGY_TOL * max(1.0, abs(ref))
        assert abs(got[name] - ref) <= tol, (name, got[name], ref)


@pytest.mark.parametrize("n,seed", [(60, 1), (300, 2), (800, 3)])
def test_go_protein_forces_energies(gpu, n, seed):
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.go_protein(n, seed)
    system, ctx = _ctx(gpu, spec)
    f, etot = ctx.getState()
    f_ref, e_ref = oracle.evaluate(spec)
    assert rel_force_err(f, f_ref) <= FORCE_TOL
    assert rms_rel_err(f, f_ref) <= 1e-5
    _check_energies(e_ref, _group_energy_map(system, ctx.getGroupEnergies()))
    assert abs(etot - sum(e_ref.values())) <= ENERGY_TOL * max(1.0, abs(sum(e_ref.values())))


@pytest.mark.parametrize("chains,length,box,seed", [(6, 50, (12.0, 12.0, 30.0), 4),
                                                    (30, 100, (15.0, 15.0, 60.0), 5)])
def test_hps_slab_forces_energies(gpu, chains, length, box, seed):
    """Periodic HPS + DH system; the second case has > 2048 beads and runs
    the column-sorted cluster layout and the charged rows."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.hps_slab(chains, length, box, slab_width=box[2] / 3, seed=seed)
    system, ctx = _ctx(gpu, spec)
    f, _ = ctx.getState(energy=False)
    f_ref, e_ref = oracle.evaluate(spec)
    assert rel_force_err(f, f_ref) <= FORCE_TOL
    _check_energies(e_ref, _group_energy_map(system, ctx.getGroupEnergies()))
    assert ctx.stats()["reordered"] == int(spec.n > 2048)
    assert ctx.stats()["charged_split"] == int(spec.n > 2048)  # DH on its own charged-pair list


@pytest.mark.parametrize("kind", ["go", "hps"])
def test_group_masks(gpu, kind):
    """getState(groups=1<<g) returns exactly that group's forces and energy
    (Observer.cpp:339-341 queries one group at a time); the HPS slab case
    runs Debye-Hueckel on the separate charged-pair list."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = (synth.go_protein(200, 9) if kind == "go"
            else synth.hps_slab(30, 100, (15.0, 15.0, 60.0), slab_width=20.0, seed=8))
    system, ctx = _ctx(gpu, spec)
    _, e_ref = oracle.evaluate(spec)
    total_f = np.zeros((spec.n, 3))
    for g, name in enumerate(system.group_names()):
        f, e = ctx.getState(groups=1 << g)
        total_f += f
        assert abs(e - e_ref[name]) <= ENERGY_TOL * max(1.0, abs(e_ref[name])), name
    f_all, _ = ctx.getState()
    assert np.allclose(total_f, f_all, rtol=0, atol=1e-6 * np.abs(f_all).max())


def test_pair_set_bit_exact(gpu):
    """The pairs the tile list makes the kernel test within the cutoff the
    tiles serve equal a brute-force enumeration with the kernel's arithmetic
    (cluster-anchored FP32 offsets, the anchor shift rounded once from FP64,
    canonical r^2); with a separate charged-pair list (Debye-Hueckel cutoff
    well above the others) its pairs equal the charged pairs within the
    Debye-Hueckel cutoff (float-float separations) that its exclusions keep."""
    from collections import Counter

    from opencafemol_gb300 import synth
    chain_len = 100
    spec = synth.hps_slab(30, chain_len, (15.0, 15.0, 60.0), slab_width=20.0, seed=6)
    system, ctx = _ctx(gpu, spec)
    pairs = ctx.list_pairs()  # builds the lists
    order = ctx.cluster_order()
    st = ctx.stats()
    assert st["charged_split"] == 1  # DH 3.5 nm against a 2.0 nm HPS cutoff
    assert st["tile_cutoff"] < st["max_cutoff"]
    got = Counter(map(tuple, pairs.tolist()))
    ref = Counter(brute_force_pairs(spec.pos, spec.box, st["tile_cutoff"], order=order))
    q = spec.dh.p0
    charged = ~np.isnan(q) & (np.nan_to_num(q) != 0)
    dh_excluded = lambda i, j: i // chain_len == j // chain_len and abs(i - j) <= 3  # ign_bond=3
    chg = {(i, j) for i, j in brute_force_pairs(spec.pos, spec.box, st["max_cutoff"], mask=charged)
           if not dh_excluded(i, j)}
    assert len(chg) > 1000 and st["charged_pairs"] >= len(chg)
    ref.update(chg)
    assert max(got.values()) <= 2, "a pair was evaluated more than once per list"
    assert got == ref


def _fp32_min_image(d, Lf, iLf):
    # d - L*rint(d/L) with FP32 roundings; L*k is exact for |k| <= 1, so the
    # separate rounding equals the kernel's fma
    return (d - Lf * np.rint((d * iLf).astype(np.float32))).astype(np.float32)


def _fp32_r2(d):
    # fmaf(dz, dz, fmaf(dy, dy, dx * dx)), each fma rounded once
    dx2 = (d[:, 0] * d[:, 0]).astype(np.float32)
    s1 = (d[:, 1].astype(np.float64) * d[:, 1] + dx2).astype(np.float32)
    return (d[:, 2].astype(np.float64) * d[:, 2] + s1).astype(np.float32)


def brute_force_pairs(pos, box, rc, order=None, mask=None):
    """Pairs (i < j) with FP32 r^2 < rc^2 under the kernels' arithmetic:
    with `order` (slot -> bead, -1 padding, clusters of 32) the anchored
    offsets of the tile kernel, otherwise the float-float separation of the
    charged rows; `mask` restricts both beads."""
    L = np.asarray(box, np.float64)
    iL = 1.0 / L
    x = np.asarray(pos, np.float64)
    w = x - np.floor(x * iL) * L                     # wrap_coord, FP64
    hi = w.astype(np.float32)                        # FP32 box-frame position
    Lf, iLf = L.astype(np.float32), iL.astype(np.float32)
    rc2 = np.float32(rc * rc)
    n = len(x)
    if order is not None:
        order = np.asarray(order)
        cl = np.zeros(n, np.int64)
        valid = order >= 0
        cl[order[valid]] = np.nonzero(valid)[0] // 32
        first = order.reshape(-1, 32)[:, 0]

        def minimg64(e):  # the minimum image only beyond half a box
            return np.where(np.abs(e) > 0.5 * L, e - L * np.rint(e * iL), e)
        # anchors: bounding-box centres of the offsets to each first bead
        a0 = np.full((len(first), 3), np.nan, np.float32)
        a0[first >= 0] = hi[first[first >= 0]]
        off0 = minimg64(w - a0[cl].astype(np.float64)).astype(np.float32)
        lo_b = np.full_like(a0, np.inf)
        hi_b = np.full_like(a0, -np.inf)
        np.minimum.at(lo_b, cl, off0)
        np.maximum.at(hi_b, cl, off0)
        with np.errstate(invalid="ignore"):  # padding-only clusters: NaN anchors
            anc = (a0 + np.float32(0.5) * (lo_b + hi_b).astype(np.float32)).astype(np.float32)
        off = minimg64(w - anc[cl].astype(np.float64)).astype(np.float32)
    else:
        lo = (w - hi.astype(np.float64)).astype(np.float32)
    out = set()
    for i in range(n - 1):
        if mask is not None and not mask[i]:
            continue
        if order is not None:
            A = minimg64(anc[cl[i + 1:]].astype(np.float64) - anc[cl[i]].astype(np.float64)).astype(np.float32)
            d = ((off[i + 1:] - off[i]).astype(np.float32) + A).astype(np.float32)
        else:
            d = ((hi[i + 1:] - hi[i]).astype(np.float32) + (lo[i + 1:] - lo[i]).astype(np.float32)).astype(np.float32)
        r2 = _fp32_r2(_fp32_min_image(d, Lf, iLf))
        hit = r2 < rc2
        if mask is not None:
            hit &= mask[i + 1:]
        for j in np.nonzero(hit)[0]:
            out.add((i, i + 1 + int(j)))
    return out


def test_cluster_order_deterministic(gpu):
    """Clusters are 32 consecutive beads of one x-y column sorted along z;
    the order is reproducible, covers every bead once, and each cluster's
    padding slots (a column's last cluster) come after its beads."""
    from opencafemol_gb300 import synth
    spec = synth.hps_slab(30, 100, (15.0, 15.0, 60.0), slab_width=20.0, seed=6)
    _, c1 = _ctx(gpu, spec)
    _, c2 = _ctx(gpu, spec)
    o1, o2 = c1.cluster_order(), c2.cluster_order()
    assert np.array_equal(o1, o2)
    real = o1[o1 >= 0]
    assert np.array_equal(np.sort(real), np.arange(spec.n))
    cl = o1.reshape(-1, 32)
    for row in cl:
        valid = row >= 0
        assert not np.any(valid[1:] & ~valid[:-1])
    # compact clusters: every full cluster spans far less than the box
    x = spec.pos - np.asarray(spec.box) * np.floor(spec.pos / np.asarray(spec.box))
    full = cl[(cl >= 0).all(axis=1)]
    ext = np.array([np.ptp(x[r], axis=0) for r in full])
    assert np.median(ext[:, 2]) < 4.0


@pytest.mark.parametrize("engine", ["tiles", "one_system"])
def test_langevin_one_step(gpu, engine):
    """x(t+dt), v(t+dt/2) after one step against the oracle's Langevin
    update fed with the oracle's forces and the same Philox stream (both
    engines of step)."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.go_protein(120, 11)
    system, ctx = _ctx(gpu, spec, seed=1234, engine=engine)
    rng = np.random.default_rng(0)
    v0 = rng.normal(scale=0.1, size=(spec.n, 3)).astype(np.float32).astype(np.float64)
    ctx.setVelocities(v0)
    ctx.step(1)
    x1, v1 = ctx.getPositions(), ctx.getVelocities()
    f_ref, _ = oracle.evaluate(spec)
    xr, vr = oracle.langevin_step(spec.pos, v0, f_ref, spec.masses, spec.temperature, spec.friction,
                                  spec.dt, 1234, 0)
    assert np.max(np.abs(v1 - vr)) <= 1e-4 * np.max(np.abs(vr))
    assert np.max(np.abs(x1 - xr)) <= 1e-6


@pytest.mark.parametrize("engine", ["tiles", "one_system"])
def test_trajectory_deterministic(gpu, engine):
    from opencafemol_gb300 import synth
    spec = synth.go_protein(150, 12)
    runs = []
    for _ in range(2):
        _, ctx = _ctx(gpu, spec, seed=99, engine=engine)
        ctx.setVelocitiesToTemperature(spec.temperature, 5)
        ctx.step(200)
        runs.append(ctx.getPositions())
    assert np.array_equal(runs[0], runs[1])


@pytest.mark.parametrize("engine", ["tiles", "one_system"])
def test_temperature_equilibrates(gpu, engine):
    """<KE> -> 3N/2 kT for Langevin dynamics at the bath temperature."""
    from opencafemol_gb300 import synth
    spec = synth.go_protein(200, 13)
    spec.friction = 1.0
    _, ctx = _ctx(gpu, spec, seed=3, engine=engine)
    ctx.setVelocitiesToTemperature(spec.temperature, 4)
    ctx.step(2000)
    kes = []
    for _ in range(60):
        ctx.step(50)
        kes.append(ctx.getKineticEnergy())
    kT = 0.00831446261815324 * spec.temperature
    expect = 1.5 * spec.n * kT
    assert abs(np.mean(kes) / expect - 1.0) < 0.05


def test_long_run_stays_finite_and_rebuilds(gpu):
    from opencafemol_gb300 import synth
    spec = synth.hps_slab(30, 100, (15.0, 15.0, 60.0), slab_width=20.0, seed=8)
    _, ctx = _ctx(gpu, spec, seed=21)
    ctx.setVelocitiesToTemperature(spec.temperature, 22)
    ctx.step(500)
    x = ctx.getPositions()
    assert np.all(np.isfinite(x))
    st = ctx.stats()
    assert st["steps_done"] == 500 and st["list_builds"] >= 500 // max(1, st["rebuild_interval"])


def test_first_evaluation_after_list_growth(gpu):
    """An 8,000-bead slab outgrows the initial tile and mask capacity on the
    first evaluation: the forces of that evaluation, of a repeated one and
    of one after dynamics all match the oracle (a regrown buffer must be
    rebuilt before use)."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.hps_slab(40, 200, (15.0, 15.0, 150.0), slab_width=30.0, seed=31)
    system, ctx = _ctx(gpu, spec)
    f1, _ = ctx.getState(energy=False)
    f2, _ = ctx.getState(energy=False)
    assert np.array_equal(f1, f2)
    f_ref, _ = oracle.evaluate(spec, cells=1)
    assert rel_force_err(f1, f_ref) <= FORCE_TOL
    ctx.step(300)
    # the kernels compute pairs from FP32 box-frame coordinates: hand both
    # sides the same FP32-exact configuration
    L = np.array(spec.box)
    x = ctx.getPositions()
    x = (x - L * np.floor(x / L)).astype(np.float32).astype(np.float64)
    x = np.where(x >= L, x - L, x)
    ctx.setPositions(x)
    f3, _ = ctx.getState(energy=False)
    f_ref3, _ = oracle.evaluate(spec, pos=x, cells=1)
    assert rel_force_err(f3, f_ref3) <= FORCE_TOL


def test_lj_same_sigma_path_bit_identical(gpu):
    """When both HPS terms carry the same per-particle sigma the kernel forms
    the sigma mixing and the s^6, s^12 powers once per pair.  Perturbing one
    bead's attractive sigma selects the general path; every bead out of that
    bead's reach gets bit-identical forces from both."""
    from opencafemol_gb300 import synth
    spec = synth.hps_slab(30, 100, (15.0, 15.0, 60.0), slab_width=20.0, seed=12)
    _, ctx = _ctx(gpu, spec)
    f_same, _ = ctx.getState(energy=False)
    k = int(np.argmin(spec.lja.p1))
    spec.lja.p1 = spec.lja.p1.copy()
    spec.lja.p1[k] *= 1.000001
    _, ctx2 = _ctx(gpu, spec)
    f_gen, _ = ctx2.getState(energy=False)
    L = np.asarray(spec.box)
    d = spec.pos - spec.pos[k]
    d -= L * np.rint(d / L)
    far = np.linalg.norm(d, axis=1) > 2.5
    assert far.sum() > 0.9 * spec.n
    assert np.array_equal(f_same[far], f_gen[far])
    assert not np.array_equal(f_same[k], f_gen[k])


def test_one_system_engine_is_the_batched_kernel(gpu):
    """A small non-periodic context steps on the batched kernel by default:
    the trajectory equals a one-slot batch's bit for bit, does not depend
    on how the steps are chunked into step calls, and evaluations between
    step calls see the current state."""
    from opencafemol_gb300 import synth
    spec = synth.go_protein(180, 14)
    system = synth.build_system(spec)
    v0 = np.random.default_rng(3).normal(scale=0.2, size=(spec.n, 3)).astype(np.float32).astype(np.float64)
    b = gpu.Batch(max_systems=1, max_total_beads=256, max_beads_per_system=256)
    slot = b.admit(system, spec.pos, velocities=v0, temperature=spec.temperature, friction=spec.friction,
                   step_size=spec.dt, seed=41, n_steps=300)
    b.run(300)
    runs = []
    for chunks in ([300], [1, 99, 200]):
        ctx = gpu.Context(system, gpu.LangevinIntegrator(spec.temperature, spec.friction, spec.dt, 41))
        ctx.setPositions(spec.pos)
        ctx.setVelocities(v0)
        for c in chunks:
            ctx.step(c)
            f, e = ctx.getState()
            assert np.all(np.isfinite(f)) and np.isfinite(e)
        st = ctx.stats()
        assert st["one_system"] == 1 and st["steps_done"] == 300
        runs.append((ctx.getPositions(), ctx.getVelocities()))
    for x, v in runs:
        assert np.array_equal(x, b.positions(slot)) and np.array_equal(v, b.velocities(slot))


def test_engine_choice(gpu):
    """Periodic systems and systems above 512 beads stay on the tiles by
    default; the one-system kernel refuses periodic systems."""
    from opencafemol_gb300 import synth
    big = synth.go_protein(600, 15)
    _, ctx = _ctx(gpu, big, engine="auto")
    ctx.step(5)
    assert ctx.stats()["one_system"] == 0
    ctx.set_engine("one_system")
    ctx.step(5)
    assert ctx.stats()["one_system"] == 1 and ctx.stats()["steps_done"] == 10
    slab = synth.hps_slab(4, 50, (12.0, 12.0, 30.0), slab_width=10.0, seed=17)
    _, cp = _ctx(gpu, slab, engine="auto")
    cp.step(3)
    assert cp.stats()["one_system"] == 0
    with pytest.raises(gpu.OCMError) as ei:
        cp.set_engine("one_system")
    assert ei.value.code == 6
