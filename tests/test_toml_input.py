"""The TOML reader: unit conversions, defaults and term selection of the
reference's reader (src/input/ReadTOMLInput.cpp,
src/input/ReadTOMLForceFieldGenerator.cpp) on small hand-written inputs."""
import math

import numpy as np
import pytest

BASE = """
[files]
output.prefix = "t"
[platform]
name = "CUDA"
[simulator]
boundary_type = "Unlimited"
delta_t = 0.2
total_step = 100
save_step = 10
seed = 7
[[systems]]
attributes.temperature = 310.0
attributes.ionic_strength = 0.2
particles = [
  {m = 100.0, pos = [0.0, 0.0, 0.0], vel = [1.0, 0.0, 0.0], group = "A"},
  {m = 110.0, pos = [3.8, 0.0, 0.0], vel = [0.0, 1.0, 0.0], group = "A"},
  {m = 120.0, pos = [3.8, 3.8, 0.0], vel = [0.0, 0.0, 1.0], group = "A"},
  {m = 130.0, pos = [3.8, 3.8, 3.8], vel = [0.0, 0.0, 0.0], group = "A"},
  {m = 140.0, pos = [7.6, 3.8, 3.8], vel = [0.0, 0.0, 0.0], group = "A"},
]
[[forcefields]]
[[forcefields.local]]
interaction = "BondLength"
potential = "Harmonic"
topology = "bond"
parameters = [
  {indices = [0, 1], v0 = 3.8, k = 110.0},
  {indices = [1, 2], v0 = 3.8, k = 110.0},
  {indices = [2, 3], v0 = 3.8, k = 110.0},
  {indices = [3, 4], v0 = 3.8, k = 110.0},
]
[[forcefields.local]]
interaction = "BondLength"
potential = "GoContact"
topology = "contact"
parameters = [{indices = [0, 4], v0 = 6.5, k = 0.5}]
[[forcefields.local]]
interaction = "BondAngle"
potential = "FlexibleLocalAngle"
topology = "none"
parameters = [
  {indices = [0, 1, 2], k = 1.0, y = "y1_PHE", d2y = "y2_PHE"},
  {indices = [1, 2, 3], k = 2.0, y = "y1_GLY", d2y = "y2_GLY"},
]
[[forcefields.local]]
interaction = "DihedralAngle"
potential = "FlexibleLocalDihedral"
topology = "none"
parameters = [
  {indices = [0, 1, 2, 3], k = 1.0, coef = "GLY-PRO"},
  {indices = [1, 2, 3, 4], k = 1.5, coef = "ALA-VAL"},
]
[[forcefields.global]]
interaction = "Pair"
potential = "ExcludedVolume"
ignore.particles_within.bond = 3
ignore.particles_within.contact = 1
epsilon = 0.6
parameters = [
  {index = 0, radius = 2.0}, {index = 1, radius = 2.5}, {index = 2, radius = 3.0},
  {index = 3, radius = 2.0}, {index = 4, radius = 2.2},
]
[[forcefields.global]]
interaction = "Pair"
potential = "DebyeHuckel"
ignore.particles_within.bond = 3
parameters = [{index = 0, charge = 1.0}, {index = 4, charge = -1.0}]
"""


def _read(text=BASE, strict=True):
    from opencafemol_gb300 import toml_input
    return toml_input.read_toml(text.encode(), strict=strict)


def test_units_and_defaults():
    from opencafemol_gb300 import toml_input
    t = _read()
    s = t.spec
    caf = math.sqrt(1 / 4.184) * 0.1
    assert toml_input.CAFETIME_PS == pytest.approx(caf, rel=1e-15)
    assert s.n == 5 and not s.periodic
    assert np.allclose(s.pos[1], [0.38, 0.0, 0.0], rtol=0, atol=1e-7)
    assert s.masses.tolist() == [100.0, 110.0, 120.0, 130.0, 140.0]
    # k (r - v0)^2 in kcal/mol/A^2 -> 1/2 k' (r - v0)^2 in kJ/mol/nm^2
    assert s.bond_k[0] == pytest.approx(110.0 * 4.184 * 100 * 2)
    assert s.bond_v0[0] == pytest.approx(0.38)
    assert s.go_k[0] == pytest.approx(0.5 * 4.184) and s.go_r0[0] == pytest.approx(0.65)
    assert s.fla_k.tolist() == pytest.approx([4.184, 2 * 4.184])
    assert s.dt == pytest.approx(0.2 * caf)
    assert s.friction == pytest.approx(0.01 / caf)  # gamma_t default
    assert t.velocities[0, 0] == pytest.approx(0.1 / caf)
    assert s.temperature == 310.0 and t.seed == 7
    assert s.exv.ratio == 2.0 and s.exv.eps == pytest.approx(0.6 * 4.184)
    assert (s.exv.ign_bond, s.exv.ign_contact) == (3, 1)
    assert s.exv.p0[2] == pytest.approx(0.3)
    assert s.dh.ratio == 5.5 and s.dh.ionic_strength == 0.2 and s.dh.temperature == 310.0
    assert np.isnan(s.dh.p0[1]) and s.dh.p0[4] == -1.0


def test_residue_selection():
    from opencafemol_gb300.forcefield import AMINO_ACIDS
    s = _read().spec
    assert [AMINO_ACIDS[a] for a in s.fla_aa] == ["PHE", "GLY"]
    assert [AMINO_ACIDS[a] for a in s.fld_aa1] == ["GLY", "ALA"]
    assert [AMINO_ACIDS[a] for a in s.fld_aa2] == ["PRO", "VAL"]


def test_gly_pro_dihedral_counted_twice():
    """A GLY-PRO coef is picked by the GLY-PRO class and by the R2-PRO
    class of the reader (ReadTOMLForceFieldGenerator.cpp:675-716)."""
    from opencafemol_gb300 import synth
    s = _read().spec
    system = synth.build_system(s)
    fld_terms = sum(f["terms"] for f in system.describe()["forces"] if f["name"].startswith("FlexibleLocalDihedral"))
    assert fld_terms == 3


def test_periodic_box():
    text = BASE.replace('boundary_type = "Unlimited"', 'boundary_type = "PeriodicCuboid"').replace(
        "attributes.temperature = 310.0",
        "attributes.temperature = 310.0\nboundary_shape.lower = [0.0, 0.0, 0.0]\n"
        "boundary_shape.upper = [100.0, 120.0, 140.0]")
    s = _read(text).spec
    assert s.periodic and s.box == pytest.approx((10.0, 12.0, 14.0), rel=1e-7)


def test_unsupported_terms():
    text = BASE + """
[[forcefields.local]]
interaction = "DihedralAngle"
potential = "Cosine"
topology = "none"
parameters = [{indices = [0, 1, 2, 3], v0 = -1.0, k = -4.0, n = 7}]
"""
    with pytest.raises(ValueError, match="Cosine"):
        _read(text)
    t = _read(text, strict=False)
    assert t.skipped == ["local force DihedralAngle/Cosine is not covered"]


def test_gaussian_terms():
    """AICG2+ Gaussian bond (v0, sigma in Angstrom) and dihedral (v0, sigma
    in radians; the sigma key may be spelled "σ")."""
    text = BASE + """
[[forcefields.local]]
interaction = "BondLength"
potential = "Gaussian"
topology = "none"
parameters = [{indices = [0, 2], v0 = 6.9701, k = -1.3709, "σ" = 0.15}]
[[forcefields.local]]
interaction = "DihedralAngle"
potential = "Gaussian"
topology = "none"
parameters = [{indices = [0, 1, 2, 3], v0 = -2.2089, k = -0.435, sigma = 0.15}]
"""
    from opencafemol_gb300 import synth
    s = _read(text).spec
    assert s.gb_idx.tolist() == [[0, 2]]
    assert s.gb_k[0] == pytest.approx(-1.3709 * 4.184) and s.gb_v0[0] == pytest.approx(0.69701)
    assert s.gb_sigma[0] == pytest.approx(0.015)
    assert s.gd_idx.tolist() == [[0, 1, 2, 3]]
    assert s.gd_k[0] == pytest.approx(-0.435 * 4.184) and s.gd_theta0[0] == -2.2089
    assert s.gd_sigma[0] == 0.15
    names = synth.build_system(s).group_names()
    assert "GaussianBond" in names and "GaussianDihedral" in names


def test_index_out_of_range():
    text = BASE.replace("{indices = [3, 4], v0 = 3.8, k = 110.0}", "{indices = [3, 5], v0 = 3.8, k = 110.0}")
    with pytest.raises(ValueError, match="exceeds the system's largest index 4"):
        _read(text)


def test_read_system_matches_oracle_energies():
    """The read system evaluates identically through the C ABI's host
    logic and the oracle (derived cutoffs, exclusions, groups)."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    s = _read().spec
    system = synth.build_system(s)
    _, e = oracle.evaluate(s)
    names = system.group_names()
    for k, v in e.items():
        if v != 0.0:
            assert k in names


def test_capped_go_wca_and_uniform_tables():
    """CappedGoContact (default capping ratio 0.75, k kcal/mol, v0 Angstrom),
    WCA with per-particle sigma / epsilon (Angstrom, kcal/mol), and the
    uniform table form of the attractive Lennard-Jones between two named
    particle sets (ReadTOMLInput.cpp:212-218, 435-621)."""
    from opencafemol_gb300 import synth
    text = BASE + """
[[forcefields.local]]
interaction = "BondLength"
potential = "CappedGoContact"
topology = "contact"
parameters = [{indices = [0, 3], v0 = 5.5, k = 0.7}, {indices = [1, 4], v0 = 6.0, k = 0.3}]
[[forcefields.global]]
interaction = "Pair"
potential = "WCA"
ignore.particles_within.bond = 1
parameters = [
  {index = 0, sigma = 4.0, epsilon = 0.2}, {index = 1, "σ" = 5.0, "ε" = 0.3},
  {index = 2, sigma = 4.5, epsilon = 0.25}, {index = 3, sigma = 4.0, epsilon = 0.2},
  {index = 4, sigma = 6.0, epsilon = 0.1},
]
[[forcefields.global]]
interaction = "Pair"
potential = "LennardJonesAttractive"
cutoff = 3.0
ignore.particles_within.bond = 1
table.A.B = {sigma = 5.0, epsilon = 0.4}
table.A.C = {sigma = 5.0, epsilon = 0.4}
parameters = [
  {index = 0, name = "A"}, {index = 1, name = "A"}, {index = 2, name = "B"},
  {index = 3, name = "B"}, {index = 4, name = "A"},
]
"""
    t = _read(text)
    s = t.spec
    assert s.cgo_topology == "contact"
    assert np.allclose(s.cgo_cap, 0.75) and np.allclose(s.cgo_r0, [0.55, 0.6])
    assert np.allclose(s.cgo_k, [0.7 * 4.184, 0.3 * 4.184])
    assert s.ljr.kind == "wca" and np.allclose(s.ljr.p1, [0.4, 0.5, 0.45, 0.4, 0.6])
    assert np.allclose(s.ljr.p0, np.array([0.2, 0.3, 0.25, 0.2, 0.1]) * 4.184)
    # A-C has no C particle and is skipped; A-B remains
    assert s.lja.kind == "uniform" and s.lja.ratio == 3.0
    assert s.lja.side.tolist() == [1, 1, 2, 2, 1]
    assert np.allclose(s.lja.p1, 0.5) and np.allclose(s.lja.p0, 0.4 * 4.184)
    names = synth.build_system(s).group_names()
    assert {"CappedGoContact", "WeeksChandlerAndersen", "UniformLennardJonesAttractive"} <= set(names)
    # two interacting pair types would need two pair slots
    two = text.replace('table.A.C = {sigma = 5.0, epsilon = 0.4}', 'table.B.B = {sigma = 5.0, epsilon = 0.4}')
    with pytest.raises(ValueError, match="2 interacting pair types"):
        _read(two)


def test_group_based_ignores():
    """ignore.group.inter / intra (ReadTOMLForceFieldGenerator.cpp:1016-1050)
    reach the generators and the oracle alike."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    text = BASE.replace('vel = [0.0, 0.0, 1.0], group = "A"}', 'vel = [0.0, 0.0, 1.0], group = "B"}') + """
[[forcefields.global]]
interaction = "Pair"
potential = "ExcludedVolume"
epsilon = 0.6
ignore.particles_within.bond = 1
ignore.group.inter = [["A", "B"]]
ignore.group.intra = ["B"]
parameters = [
  {index = 0, radius = 2.0}, {index = 1, radius = 2.0}, {index = 2, radius = 2.0},
  {index = 3, radius = 2.0}, {index = 4, radius = 2.0},
]
"""
    t = _read(text)
    s = t.spec
    assert s.exv.ignore_groups == [("A", "B"), ("B", "B")]
    assert s.group_names == ["A", "A", "B", "A", "A"]
    d = synth.build_system(s).describe()["forces"]
    exv = next(f for f in d if f["name"] == "ExcludedVolume")
    # (others, others), (A, others), (A, A), (B, others); A-B and B-B ignored
    # (the sides without particles add no pair, as in the reference)
    assert exv["interaction_groups"] == 4
    _, e = oracle.evaluate(s, fp32_cutoff=False)
    # only A-A pairs beyond one bond remain: (0, 3), (0, 4), (1, 3), (1, 4)
    x = s.pos
    rc = 2.0 * 0.4
    want = 0.6 * 4.184 * sum(0.4 ** 12 * (np.linalg.norm(x[i] - x[j]) ** -12 - rc ** -12)
                             for i, j in [(0, 3), (0, 4), (1, 3), (1, 4)]
                             if np.linalg.norm(x[i] - x[j]) < rc)
    assert e["ExcludedVolume"] == pytest.approx(want, rel=1e-12, abs=1e-12)


def test_molecule_based_ignores():
    """ignore.molecule = "Intra": no pair inside a bond-connected molecule;
    pairs between molecules interact (ReadTOMLForceFieldGenerator.cpp:963-985,
    molecules from the bond edges, ReadTOMLInput.cpp:405)."""
    from opencafemol_gb300 import synth
    from oracle import oracle
    # two chains: 0-1-2 and 3-4 (drop the 2-3 bond of BASE)
    text = BASE.replace("  {indices = [2, 3], v0 = 3.8, k = 110.0},\n", "") + """
[[forcefields.global]]
interaction = "Pair"
potential = "ExcludedVolume"
epsilon = 0.6
ignore.molecule = "Intra"
parameters = [
  {index = 0, radius = 2.5}, {index = 1, radius = 2.5}, {index = 2, radius = 2.5},
  {index = 3, radius = 2.5}, {index = 4, radius = 2.5},
]
"""
    s = _read(text).spec
    assert s.exv.ign_molecule
    names = [f["name"] for f in synth.build_system(s).describe()["forces"]]
    assert "ExcludedVolume" in names
    _, e = oracle.evaluate(s, fp32_cutoff=False)
    x = s.pos
    rc = 2.0 * 0.5
    want = 0.6 * 4.184 * sum(0.5 ** 12 * (np.linalg.norm(x[i] - x[j]) ** -12 - rc ** -12)
                             for i in (0, 1, 2) for j in (3, 4) if np.linalg.norm(x[i] - x[j]) < rc)
    assert want != 0.0
    assert e["ExcludedVolume"] == pytest.approx(want, rel=1e-12)


def test_molecule_ignore_list_from_topology():
    """The host builds the molecule ignore list from the bond edges."""
    from opencafemol_gb300 import synth
    topo = synth.Topology(5)
    topo.add_edges(np.array([[0, 1], [1, 2], [3, 4]]), "bond")
    pairs = synth._ignore(topo, -1, -1, True)
    assert sorted(map(tuple, pairs.tolist())) == [(0, 1), (0, 2), (1, 2), (3, 4)]


def test_env_named_parameters():
    """A parameter written as a string names an entry of the block's env
    table (Utility.hpp:33-139); table names (y, coef) stay strings."""
    text = BASE + """
[[forcefields.global]]
interaction = "Pair"
potential = "ExcludedVolume"
epsilon = 0.6
env.R = 2.0
env.OFF = 1
ignore.particles_within.bond = 1
parameters = [
  {index = 0, radius = "R"}, {index = 0, offset = "OFF", radius = 1.5}, {index = 2, radius = "R"},
  {index = 3, radius = 2.0}, {index = 4, radius = "R"},
]
"""
    s = _read(text).spec
    assert np.allclose(s.exv.p0, [0.2, 0.15, 0.2, 0.2, 0.2])
    bad = text.replace('env.R = 2.0\n', '')
    with pytest.raises(ValueError, match='named variable "R"'):
        _read(bad)
    # offset is optional (find_parameter_or, Utility.hpp:140-155): a name
    # that env does not define falls back to 0 instead of failing
    lenient = text.replace('env.OFF = 1\n', '')
    s = _read(lenient).spec
    assert np.allclose(s.exv.p0, [0.15, np.nan, 0.2, 0.2, 0.2], equal_nan=True)
