"""The reference's force-field variants on the GPU against the FP64 oracle:
WeeksChandlerAndersen (geometric epsilon mean, in the repulsive
Lennard-Jones slot), the uniform attractive Lennard-Jones and uniform WCA
between two particle lists, and capped Go contacts, on the batched and the
plain engine (non-periodic and periodic).

Tolerances as everywhere: per-bead force error <= 1e-4 relative to
max(|F_i|, 1e-3 F_rms); per-term energies <= 1e-5 relative."""
import numpy as np
import pytest

from conftest import rel_force_err

pytestmark = pytest.mark.gpu


def _with_variants(spec, seed, uniform_wca=False):
    """Add WCA (or uniform WCA), uniform LJA between two halves, and capped
    Go contacts, some of them compressed below cap r0."""
    from opencafemol_gb300 import synth
    rng = np.random.default_rng(seed)
    n = spec.n
    side = np.zeros(n, np.int8)
    side[: n // 2] |= 1
    side[n // 3:] |= 2
    if uniform_wca:
        spec.ljr = synth.PairTerm(ratio=0.0, p0=np.full(n, 0.9), p1=np.full(n, 0.58), kind="uniform",
                                  side=side, ign_bond=1)
    else:
        spec.ljr = synth.PairTerm(ratio=0.0, p0=rng.uniform(0.3, 1.5, n), p1=rng.uniform(0.35, 0.55, n),
                                  kind="wca", ign_bond=1)
    spec.lja = synth.PairTerm(ratio=3.0, p0=np.full(n, 0.6), p1=np.full(n, 0.5), kind="uniform", side=side,
                              ign_bond=1)
    pairs = rng.choice(n, size=(n // 4, 2))
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    d = spec.pos[pairs[:, 1]] - spec.pos[pairs[:, 0]]
    if spec.periodic:
        L = np.asarray(spec.box)
        d -= L * np.rint(d / L)
    r = np.linalg.norm(d, axis=1)
    keep = r < 3.0
    spec.cgo_idx = pairs[keep]
    spec.cgo_r0 = r[keep] * rng.uniform(0.9, 1.6, keep.sum())  # r / r0 below 0.8 for part of them
    spec.cgo_k = rng.uniform(0.5, 2.0, keep.sum())
    spec.cgo_cap = 0.8
    assert np.any(r[keep] / spec.cgo_r0 < spec.cgo_cap) and np.any(r[keep] / spec.cgo_r0 > spec.cgo_cap)
    return spec


def _check(system, f, e32, f_ref, e_ref):
    assert rel_force_err(f, f_ref) <= 1e-4
    for g, name in enumerate(system.group_names()):
        assert abs(e32[g] - e_ref[name]) <= 1e-5 * max(1.0, abs(e_ref[name])), name


@pytest.mark.parametrize("uniform_wca", [False, True])
def test_variants_batched_and_plain(gpu, uniform_wca):
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = _with_variants(synth.go_protein(400, 77), seed=5, uniform_wca=uniform_wca)
    system = synth.build_system(spec)
    names = system.group_names()
    assert "CappedGoContact" in names and "UniformLennardJonesAttractive" in names
    assert ("UniformWeeksChadlerAndersen" if uniform_wca else "WeeksChandlerAndersen") in names
    f_ref, e_ref = oracle.evaluate(spec)
    b = gpu.Batch(max_systems=1, max_total_beads=512, max_beads_per_system=512)
    slot = b.admit(system, spec.pos, seed=1, n_steps=1)
    f, e32 = b.state(slot)
    _check(system, f, e32, f_ref, e_ref)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 1))
    ctx.setPositions(spec.pos)
    fp, _ = ctx.getState()
    _check(system, fp, ctx.getGroupEnergies(), f_ref, e_ref)


def test_variants_periodic_plain(gpu):
    """A periodic slab of 3,000 beads (cluster layout, charged rows) with WCA
    in place of the HPS repulsion and the uniform attraction."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = _with_variants(synth.hps_slab(30, 100, (15.0, 15.0, 60.0), slab_width=20.0, seed=21), seed=6)
    system = synth.build_system(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 1))
    ctx.setPositions(spec.pos)
    f, _ = ctx.getState()
    assert ctx.stats()["reordered"] == 1
    f_ref, e_ref = oracle.evaluate(spec)
    _check(system, f, ctx.getGroupEnergies(), f_ref, e_ref)


def test_toml_variants_match_oracle(gpu):
    """The variants as the TOML reader builds them (capped Go contacts as
    "contact" edges of the topology, WCA, a uniform table pair) on a
    60-bead chain."""
    from opencafemol_gb300 import synth
    from opencafemol_gb300.toml_input import read_toml
    from oracle import oracle
    base = synth.go_protein(60, 40)
    rng = np.random.default_rng(40)
    parts = ",\n".join(f'  {{m = 120.0, pos = [{x[0] * 10:.4f}, {x[1] * 10:.4f}, {x[2] * 10:.4f}]}}'
                       for x in base.pos)
    bonds = ",\n".join(f"  {{indices = [{i}, {i + 1}], v0 = 3.8, k = 110.0}}" for i in range(59))
    cgo = ",\n".join(f"  {{indices = [{i}, {i + 5}], v0 = {rng.uniform(5, 9):.3f}, k = 0.6}}"
                     for i in range(0, 50, 3))
    wca = ",\n".join(f'  {{index = {i}, sigma = {rng.uniform(3.5, 5.5):.3f}, epsilon = 0.3}}' for i in range(60))
    names = ",\n".join(f'  {{index = {i}, name = "{"A" if i % 2 else "B"}"}}' for i in range(60))
    text = f"""
[simulator]
boundary_type = "Unlimited"
delta_t = 0.2
total_step = 10
save_step = 10
[[systems]]
attributes.temperature = 300.0
particles = [
{parts}
]
[[forcefields]]
[[forcefields.local]]
interaction = "BondLength"
potential = "Harmonic"
topology = "bond"
parameters = [
{bonds}
]
[[forcefields.local]]
interaction = "BondLength"
potential = "CappedGoContact"
topology = "contact"
capping_ratio = 0.85
parameters = [
{cgo}
]
[[forcefields.global]]
interaction = "Pair"
potential = "WCA"
ignore.particles_within.bond = 1
ignore.particles_within.contact = 1
parameters = [
{wca}
]
[[forcefields.global]]
interaction = "Pair"
potential = "LennardJonesAttractive"
cutoff = 3.0
ignore.particles_within.bond = 2
table.A.B = {{sigma = 5.0, epsilon = 0.4}}
parameters = [
{names}
]
"""
    spec = read_toml(text.encode()).spec
    system = synth.build_system(spec)
    f_ref, e_ref = oracle.evaluate(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 1))
    ctx.setPositions(spec.pos)
    f, _ = ctx.getState()
    _check(system, f, ctx.getGroupEnergies(), f_ref, e_ref)
    assert abs(e_ref["CappedGoContact"]) > 0 and abs(e_ref["UniformLennardJonesAttractive"]) > 0


def test_group_based_ignores_both_engines(gpu):
    """Group-based ignores (ignore.group.inter / intra of the reference's
    inputs): excluded volume skips A-B pairs, Debye-Hueckel skips A-A pairs."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.go_protein(240, 91)
    spec.group_names = ["A" if i < 120 else ("B" if i < 200 else None) for i in range(spec.n)]
    spec.exv.ignore_groups = [("A", "B")]
    spec.dh.ignore_groups = [("A", "A")]
    system = synth.build_system(spec)
    f_ref, e_ref = oracle.evaluate(spec)
    b = gpu.Batch(max_systems=1, max_total_beads=256, max_beads_per_system=256)
    slot = b.admit(system, spec.pos, seed=1, n_steps=1)
    f, e32 = b.state(slot)
    _check(system, f, e32, f_ref, e_ref)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 1))
    ctx.setPositions(spec.pos)
    fp, _ = ctx.getState()
    _check(system, fp, ctx.getGroupEnergies(), f_ref, e_ref)


def test_molecule_based_ignores_both_engines(gpu):
    """ignore.molecule = "Intra": Debye-Hueckel acts only between chains."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.hps_slab(4, 50, (12.0, 12.0, 30.0), slab_width=10.0, seed=17)
    spec.dh.ign_molecule = True
    spec.dh.ign_bond = -1
    system = synth.build_system(spec)
    f_ref, e_ref = oracle.evaluate(spec)
    ctx = gpu.Context(system, gpu.LangevinIntegrator(300.0, 0.1, 0.01, 1))
    ctx.setPositions(spec.pos)
    fp, _ = ctx.getState()
    _check(system, fp, ctx.getGroupEnergies(), f_ref, e_ref)
