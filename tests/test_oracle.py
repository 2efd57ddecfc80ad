"""Known-answer tests that pin the FP64 oracle (the reference ships no
golden vectors, so these analytic identities are the pin)."""
import copy
import math

import numpy as np
import pytest

import opencafemol_gb300 as ocm
from opencafemol_gb300 import synth
from oracle import oracle

KCAL = 4.184


def two_bead(r, **terms):
    """Two beads at distance r along x with the given single term."""
    s = synth.CGSpec(n=2, pos=np.array([[0.0, 0, 0], [r, 0, 0]]), masses=np.ones(2))
    for k, v in terms.items():
        setattr(s, k, v)
    return s


def test_go_minimum():
    eps, r0 = 2.0, 0.55
    s = two_bead(r0)
    s.contacts = np.array([[0, 1]])
    s.go_k, s.go_r0 = np.array([eps]), np.array([r0])
    f, e = oracle.evaluate(s, fp32_cutoff=False)
    assert e["GoContact"] == pytest.approx(-eps, rel=1e-14)
    assert np.abs(f).max() < 1e-12


def test_exv_and_dh_vanish_at_cutoff():
    rad = np.array([0.3, 0.35])
    exv = synth.PairTerm(ratio=2.0, p0=rad, eps=1.0)
    rc = 2.0 * 0.65
    s = two_bead(rc * (1 - 1e-9), exv=exv)
    _, e = oracle.evaluate(s, fp32_cutoff=False)
    assert abs(e["ExcludedVolume"]) < 1e-10
    s = two_bead(rc * 1.000001, exv=exv)
    _, e = oracle.evaluate(s, fp32_cutoff=False)
    assert e["ExcludedVolume"] == 0.0
    dh = synth.PairTerm(ratio=3.0, p0=np.array([1.0, -1.0]), ionic_strength=0.15, temperature=300)
    p = oracle.dh_params(0.15, 300, 3.0)
    s = two_bead(p["cutoff"] * (1 - 1e-10), dh=dh)
    _, e = oracle.evaluate(s, fp32_cutoff=False)
    assert abs(e["DebyeHuckel"]) < 1e-10


def test_lj_repulsive_continuity():
    sig = np.array([0.6, 0.6])
    t = 2 ** (1 / 6) * 0.6
    ljr = synth.PairTerm(ratio=4.0, p0=np.array([1.0, 1.0]), p1=sig)
    for r in (t * (1 - 1e-9), t * (1 + 1e-9)):
        f, e = oracle.evaluate(two_bead(r, ljr=ljr), fp32_cutoff=False)
        assert abs(e["LennardJonesRepulsive"]) < 1e-7
        assert np.abs(f).max() < 1e-5


def test_lj_attractive_plateau_and_switch():
    sig = np.array([0.6, 0.6])
    lja = synth.PairTerm(ratio=3.0, p0=np.array([0.8, 0.8]), p1=sig)
    _, e = oracle.evaluate(two_bead(0.5, lja=lja), fp32_cutoff=False)
    assert e["LennardJonesAttractive"] == pytest.approx(-0.8, rel=1e-14)
    rc = 0.6 * 3.0
    _, e = oracle.evaluate(two_bead(rc * (1 - 1e-9), lja=lja), fp32_cutoff=False)
    assert abs(e["LennardJonesAttractive"]) < 1e-12
    # inside the switching region the energy is the LJ value times S(x)
    r = 0.95 * rc
    x = (r - 0.9 * rc) / (0.1 * rc)
    sw = 1 - 10 * x ** 3 + 15 * x ** 4 - 6 * x ** 5
    lj = 4 * 0.8 * ((0.6 / r) ** 12 - (0.6 / r) ** 6)
    _, e = oracle.evaluate(two_bead(r, lja=lja), fp32_cutoff=False)
    assert e["LennardJonesAttractive"] == pytest.approx(lj * sw, rel=1e-12)


def _angle_spec(theta, aa=0, k=1.0):
    p1 = np.array([0.38, 0.0, 0.0])
    p3 = 0.38 * np.array([math.cos(theta), math.sin(theta), 0.0])
    s = synth.CGSpec(n=3, pos=np.array([p1, [0, 0, 0], p3]), masses=np.ones(3))
    s.fla_idx, s.fla_k, s.fla_aa = np.array([[0, 1, 2]]), np.array([k]), np.array([aa], np.int32)
    return s


def test_fla_passes_through_nodes():
    h = (2.87979 - 1.30900) / 9
    for aa in (0, 7, 14):
        y = ocm.fla_spline_table(ocm.AMINO_ACIDS[aa])
        emin = oracle.fla_min_energy(aa)
        for k in range(1, 9):
            _, e = oracle.evaluate(_angle_spec(1.309 + h * k, aa), fp32_cutoff=False)
            assert e["FlexibleLocalAngle"] == pytest.approx(y[k] - emin, abs=1e-9)


def test_fla_walls():
    y = ocm.fla_spline_table("ALA")
    emin = oracle.fla_min_energy(0)
    for th, ref in ((1.2, 30 * (1.309 - 1.2) + y[0] - emin), (3.0, 30 * (3.0 - 2.87979) + y[9] - emin)):
        _, e = oracle.evaluate(_angle_spec(th), fp32_cutoff=False)
        assert e["FlexibleLocalAngle"] == pytest.approx(ref, rel=1e-12)


def _dihedral_spec(phi, aa1, aa2):
    # x1 along +y above x2, x2 at origin, x3 on +x, x4 rotated by phi about x
    p = np.array([[0.0, 0.38, 0.0], [0, 0, 0], [0.38, 0, 0],
                  [0.38, 0.38 * math.cos(phi), 0.38 * math.sin(phi)]])
    s = synth.CGSpec(n=4, pos=p, masses=np.ones(4))
    s.fld_idx, s.fld_k = np.array([[0, 1, 2, 3]]), np.array([1.0])
    s.fld_aa1, s.fld_aa2 = np.array([aa1], np.int32), np.array([aa2], np.int32)
    return s


def test_fld_iupac_sign_and_minimum():
    aa = list(ocm.AMINO_ACIDS)
    keys = ocm.fld_table_keys()
    a1, a2 = aa.index("ALA"), aa.index("LEU")
    c = ocm.fld_fourier_table("ALA-R3")
    emin = oracle.fld_min_energy(keys.index("ALA-R3"))
    for phi in (math.radians(60), math.radians(-100)):
        _, e = oracle.evaluate(_dihedral_spec(phi, a1, a2), fp32_cutoff=False)
        ref = (c[0] - emin + c[1] * math.cos(phi) + c[2] * math.sin(phi) + c[3] * math.cos(2 * phi)
               + c[4] * math.sin(2 * phi) + c[5] * math.cos(3 * phi) + c[6] * math.sin(3 * phi))
        assert e["FlexibleLocalDihedral"] == pytest.approx(ref, rel=1e-12)
    grid = np.linspace(-math.pi, math.pi, 20001)
    vals = [c[0] - emin + c[1] * np.cos(g) + c[2] * np.sin(g) + c[3] * np.cos(2 * g) + c[4] * np.sin(2 * g)
            + c[5] * np.cos(3 * g) + c[6] * np.sin(3 * g) for g in grid]
    assert min(vals) == pytest.approx(0.0, abs=1e-6)


def test_gly_pro_dihedral_counts_twice():
    aa = list(ocm.AMINO_ACIDS)
    keys = ocm.fld_table_keys()
    phi = 0.7
    _, e = oracle.evaluate(_dihedral_spec(phi, aa.index("GLY"), aa.index("PRO")), fp32_cutoff=False)
    tot = 0.0
    for key in ("GLY-PRO", "R2-PRO"):
        c = ocm.fld_fourier_table(key)
        emin = oracle.fld_min_energy(keys.index(key))
        tot += (c[0] - emin + c[1] * math.cos(phi) + c[2] * math.sin(phi) + c[3] * math.cos(2 * phi)
                + c[4] * math.sin(2 * phi) + c[5] * math.cos(3 * phi) + c[6] * math.sin(3 * phi))
    assert e["FlexibleLocalDihedral"] == pytest.approx(tot, rel=1e-12)


def _total_energy(spec, pos):
    _, e = oracle.evaluate(spec, fp32_cutoff=False, pos=pos)
    return sum(e.values())


@pytest.mark.parametrize("which", ["go", "hps"])
def test_forces_are_minus_gradient(which):
    if which == "go":
        spec = synth.go_protein(40, 21)
    else:
        spec = synth.hps_slab(4, 20, (9.0, 9.0, 20.0), 6.0, seed=22)
    f, _ = oracle.evaluate(spec, fp32_cutoff=False)
    rng = np.random.default_rng(0)
    h = 1e-6
    for i in rng.choice(spec.n, 8, replace=False):
        for c in range(3):
            xp, xm = spec.pos.copy(), spec.pos.copy()
            xp[i, c] += h
            xm[i, c] -= h
            fd = -(_total_energy(spec, xp) - _total_energy(spec, xm)) / (2 * h)
            assert fd == pytest.approx(f[i, c], rel=2e-5, abs=2e-4 * (1 + abs(f[i, c])))


def test_net_force_zero_and_invariance():
    spec = synth.go_protein(60, 23)
    f, e = oracle.evaluate(spec, fp32_cutoff=False)
    assert np.abs(f.sum(0)).max() < 1e-9 * np.abs(f).max()
    R = np.linalg.qr(np.random.default_rng(1).normal(size=(3, 3)))[0]
    moved = spec.pos @ R.T + np.array([3.0, -2.0, 1.0])
    f2, e2 = oracle.evaluate(spec, fp32_cutoff=False, pos=moved)
    for k in e:
        assert e2[k] == pytest.approx(e[k], rel=1e-9, abs=1e-9)
    assert np.allclose(f2, f @ R.T, atol=1e-8 * np.abs(f).max())
    hps = synth.hps_slab(4, 20, (9.0, 9.0, 20.0), 6.0, seed=24)
    fh, _ = oracle.evaluate(hps, fp32_cutoff=False)
    assert np.abs(fh.sum(0)).max() < 1e-9 * np.abs(fh).max()


def test_philox_known_answers():
    """Philox4x32-10 (the round function the engine and the oracle share)
    against the published known-answer vectors."""
    out = []
    for ctr, key, ref in (
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ):
        got = philox_words(ctr, key)
        out.append(got == ref)
    assert all(out)


def philox_words(ctr, key):
    """Pure-Python Philox4x32-10 round function (same algorithm as the
    engine and the oracle)."""
    c = list(ctr)
    k0, k1 = key
    M = 0xFFFFFFFF
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & M, p1 & M, ((p0 >> 32) ^ c[3] ^ k1) & M, p0 & M]
        k0 = (k0 + 0x9E3779B9) & M
        k1 = (k1 + 0xBB67AE85) & M
    return tuple(c)


def test_oracle_gaussian_uses_philox_words():
    seed, stream, bead, step = 1234, 0, 17, 99
    w = philox_words((bead, step & 0xFFFFFFFF, step >> 32, 0), (seed, 0x6F636D31 ^ stream))
    u = [((x >> 8) + 1) / 16777216.0 for x in w]
    ref = [math.sqrt(-2 * math.log(u[0])) * math.cos(2 * math.pi * u[1]),
           math.sqrt(-2 * math.log(u[0])) * math.sin(2 * math.pi * u[1]),
           math.sqrt(-2 * math.log(u[2])) * math.cos(2 * math.pi * u[3])]
    assert np.allclose(oracle.gaussian3(seed, stream, bead, step), ref, rtol=1e-14)


def test_langevin_friction_free_is_leapfrog():
    rng = np.random.default_rng(5)
    x, v, f = rng.normal(size=(4, 3)), rng.normal(size=(4, 3)), rng.normal(size=(4, 3))
    m = np.array([1.0, 2.0, 3.0, 4.0])
    x1, v1 = oracle.langevin_step(x, v, f, m, T=0.0, gamma=0.0, dt=0.01, seed=1, step=0)
    assert np.allclose(v1, v + 0.01 * f / m[:, None], atol=1e-14)
    assert np.allclose(x1, x + 0.01 * v1, atol=1e-14)


def test_oracle_noise_is_standard_normal():
    g = np.array([oracle.gaussian3(9, 0, b, 3) for b in range(20000)]).ravel()
    assert abs(g.mean()) < 0.02 and abs(g.std() - 1) < 0.02


@pytest.mark.parametrize("case", ["slab", "protein"])
def test_cell_grid_matches_all_pairs(case):
    """The oracle's cell-grid pair enumeration (used for large systems)
    visits exactly the pairs of the all-pairs loop."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    if case == "slab":
        spec = synth.hps_slab(12, 100, (12.0, 12.0, 40.0), slab_width=14.0, seed=21)
    else:
        spec = synth.go_protein(700, 22)
    f0, e0 = oracle.evaluate(spec, cells=0)
    f1, e1 = oracle.evaluate(spec, cells=1)
    assert np.max(np.abs(f1 - f0)) <= 1e-9 * np.abs(f0).max()
    for k in e0:
        assert abs(e1[k] - e0[k]) <= 1e-9 * max(1.0, abs(e0[k])), k


def test_gaussian_terms_at_their_centres():
    """At the structure the AICG2+ Gaussian terms are centred on, every bond
    and dihedral sits at the bottom of its well: E = sum k, zero force."""
    spec = synth.add_aicg_gaussians(synth.go_protein(30, 41), seed=42)
    only = synth.CGSpec(n=spec.n, pos=spec.pos, masses=spec.masses)
    for k in ("gb_idx", "gb_k", "gb_v0", "gb_sigma", "gd_idx", "gd_k", "gd_theta0", "gd_sigma"):
        setattr(only, k, getattr(spec, k))
    f, e = oracle.evaluate(only, fp32_cutoff=False)
    assert e["GaussianBond"] == pytest.approx(spec.gb_k.sum(), rel=1e-12)
    assert e["GaussianDihedral"] == pytest.approx(spec.gd_k.sum(), rel=1e-12)
    assert np.abs(f).max() < 1e-9


def test_gaussian_dihedral_is_periodic():
    """dphi is wrapped to [-pi, pi): a centre shifted by 2 pi is the same term."""
    spec = synth.add_aicg_gaussians(synth.go_protein(12, 43), seed=44)
    spec.gb_idx = spec.gb_idx[:0]
    x = spec.pos + np.random.default_rng(1).normal(scale=0.05, size=spec.pos.shape)
    f0, e0 = oracle.evaluate(spec, fp32_cutoff=False, pos=x)
    shifted = copy.deepcopy(spec)
    shifted.gd_theta0 = spec.gd_theta0 + 2 * math.pi
    f1, e1 = oracle.evaluate(shifted, fp32_cutoff=False, pos=x)
    assert e1["GaussianDihedral"] == pytest.approx(e0["GaussianDihedral"], rel=1e-12)
    assert np.allclose(f1, f0, rtol=1e-10, atol=1e-10)


def test_gaussian_forces_are_minus_gradient():
    spec = synth.add_aicg_gaussians(synth.go_protein(40, 45), seed=46)
    pos = spec.pos + np.random.default_rng(2).normal(scale=0.01, size=spec.pos.shape)
    f, _ = oracle.evaluate(spec, fp32_cutoff=False, pos=pos)
    rng = np.random.default_rng(3)
    h = 1e-6
    for i in rng.choice(spec.n, 8, replace=False):
        for c in range(3):
            xp, xm = pos.copy(), pos.copy()
            xp[i, c] += h
            xm[i, c] -= h
            fd = -(_total_energy(spec, xp) - _total_energy(spec, xm)) / (2 * h)
            assert fd == pytest.approx(f[i, c], rel=2e-5, abs=2e-4 * (1 + abs(f[i, c])))


# --------------------------------------------------------------------------
# WCA, uniform Lennard-Jones and capped Go (the reference's variants)
# --------------------------------------------------------------------------
def test_wca_geometric_mean_and_cutoff():
    """WeeksChandlerAndersenForceFieldGenerator.cpp:38-45: sigma arithmetic,
    epsilon geometric mean; E(sigma) = eps, E(2^(1/6) sigma) = 0; cutoff
    2^(1/6) (sigma_max + sigma_2nd) / 2."""
    sig, eps = np.array([0.5, 0.7]), np.array([1.0, 4.0])
    wca = synth.PairTerm(ratio=0.0, p0=eps, p1=sig, kind="wca")
    s = 0.6
    _, e = oracle.evaluate(two_bead(s, ljr=wca), fp32_cutoff=False)
    assert e["WeeksChandlerAndersen"] == pytest.approx(2.0, rel=1e-13)  # sqrt(1 * 4)
    t = 2 ** (1 / 6) * s
    f, e = oracle.evaluate(two_bead(t * (1 - 1e-9), ljr=wca), fp32_cutoff=False)
    assert abs(e["WeeksChandlerAndersen"]) < 1e-7 and np.abs(f).max() < 1e-5
    _, e = oracle.evaluate(two_bead(t * (1 + 1e-9), ljr=wca), fp32_cutoff=False)
    assert e["WeeksChandlerAndersen"] == 0.0


def test_uniform_pairs_only_between_former_and_latter():
    """Uniform generators act on (former, latter) pairs only."""
    n = 3
    pos = np.array([[0.0, 0, 0], [0.6, 0, 0], [0.0, 0.6, 0]])
    side = np.array([1, 2, 1], np.int8)  # 0 and 2 former, 1 latter
    lja = synth.PairTerm(ratio=3.0, p0=np.full(n, 0.5), p1=np.full(n, 0.4), kind="uniform", side=side)
    s = synth.CGSpec(n=n, pos=pos, masses=np.ones(n), lja=lja)
    _, e = oracle.evaluate(s, fp32_cutoff=False)

    def lj(r):  # below the 0.9 * 1.2 nm switch
        return 4 * 0.5 * ((0.4 / r) ** 12 - (0.4 / r) ** 6)
    # (0, 1) at 0.6 nm and (2, 1) at 0.6 sqrt(2) nm; (0, 2) are both former
    assert e["UniformLennardJonesAttractive"] == pytest.approx(lj(0.6) + lj(0.6 * np.sqrt(2)), rel=1e-12)


def test_capped_go_matches_go_above_cap_and_is_c1():
    """Capped Go: the Go 10-12 value beyond cap r0, a straight line below,
    equal value and slope at r = cap r0."""
    k, r0, cap = 1.5, 0.6, 0.8

    def energy(r):
        s = two_bead(r)
        s.cgo_idx, s.cgo_k, s.cgo_r0, s.cgo_cap = np.array([[0, 1]]), np.array([k]), np.array([r0]), cap
        f, e = oracle.evaluate(s, fp32_cutoff=False)
        return e["CappedGoContact"], f
    e_min, f_min = energy(r0)
    assert e_min == pytest.approx(-k, rel=1e-14) and np.abs(f_min).max() < 1e-12
    rb = cap * r0
    lo, _ = energy(rb * (1 - 1e-9))
    hi, _ = energy(rb * (1 + 1e-9))
    assert lo == pytest.approx(hi, rel=1e-7)
    h = 1e-6
    slope_lo = (energy(rb - h)[0] - energy(rb - 2 * h)[0]) / h
    slope_hi = (energy(rb + 2 * h)[0] - energy(rb + h)[0]) / h
    assert slope_lo == pytest.approx(slope_hi, rel=1e-4)
    # linear below the cap
    e1, e2, e3 = energy(0.2)[0], energy(0.3)[0], energy(0.4)[0]
    assert (e3 - e2) == pytest.approx(e2 - e1, rel=1e-10)


def test_variant_forces_are_minus_gradient():
    rng = np.random.default_rng(4)
    n = 6
    pos = rng.normal(scale=0.45, size=(n, 3))
    wca = synth.PairTerm(ratio=0.0, p0=rng.uniform(0.5, 2.0, n), p1=rng.uniform(0.5, 0.8, n), kind="wca")
    side = np.array([1, 1, 3, 2, 2, 3], np.int8)
    lja = synth.PairTerm(ratio=3.0, p0=np.full(n, 0.7), p1=np.full(n, 0.45), kind="uniform", side=side)
    s = synth.CGSpec(n=n, pos=pos, masses=np.ones(n), ljr=wca, lja=lja)
    s.cgo_idx = np.array([[0, 3], [1, 4], [2, 5]])
    s.cgo_k, s.cgo_r0, s.cgo_cap = np.array([1.0, 2.0, 0.5]), np.array([0.9, 0.6, 1.2]), 0.8
    f, _ = oracle.evaluate(s, fp32_cutoff=False)
    h = 1e-6
    for i in range(n):
        for c in range(3):
            xp, xm = pos.copy(), pos.copy()
            xp[i, c] += h
            xm[i, c] -= h
            ep = sum(oracle.evaluate(s, fp32_cutoff=False, pos=xp)[1].values())
            em = sum(oracle.evaluate(s, fp32_cutoff=False, pos=xm)[1].values())
            assert f[i, c] == pytest.approx(-(ep - em) / (2 * h), rel=1e-5, abs=1e-5)


def test_group_based_ignores():
    """ignore.group: pairs whose (group, group) is ignored do not interact
    (either order); particles without a group, or in a group no ignore names,
    interact with everyone."""
    pos = np.array([[0.0, 0, 0], [0.5, 0, 0], [0.0, 0.5, 0], [0.5, 0.5, 0]])
    rad = np.full(4, 0.3)
    names = ["A", "B", None, "A"]

    def energy(ignore):
        exv = synth.PairTerm(ratio=2.0, p0=rad, eps=1.0, ignore_groups=ignore)
        s = synth.CGSpec(n=4, pos=pos, masses=np.ones(4), exv=exv, group_names=names)
        return oracle.evaluate(s, fp32_cutoff=False)[1]["ExcludedVolume"]

    def pair(i, j):
        r = np.linalg.norm(pos[i] - pos[j])
        return 0.6 ** 12 * (r ** -12 - 1.2 ** -12)
    every = sum(pair(i, j) for i in range(4) for j in range(i + 1, 4))
    assert energy(None) == pytest.approx(every, rel=1e-12)
    # A-B ignored: (0, 1) and (3, 1) drop out
    assert energy([("B", "A")]) == pytest.approx(every - pair(0, 1) - pair(1, 3), rel=1e-12)
    # intra A: (0, 3) drops out
    assert energy([("A", "A")]) == pytest.approx(every - pair(0, 3), rel=1e-12)
