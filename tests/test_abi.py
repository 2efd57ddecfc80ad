"""CPU tests of the C ABI and the host-side mirror of the reference's
generators, topology and system assembly (no GPU needed)."""
import re
from pathlib import Path

import numpy as np
import pytest

import opencafemol_gb300 as ocm
from opencafemol_gb300 import synth
from oracle import oracle

HEADER = Path(__file__).resolve().parents[1] / "include" / "ocm.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"^[A-Za-z_][\w \*]*?\b(ocm_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) > 50
    for name in names:
        assert hasattr(ocm.lib, name), name


def test_abi_version_and_device_count():
    """The library reports the version the header declares (bumped whenever
    a struct or signature of the header changes)."""
    import re
    header = (Path(__file__).resolve().parents[1] / "include" / "ocm.h").read_text()
    declared = int(re.search(r"#define OCM_ABI_VERSION (\d+)", header).group(1))
    assert ocm.lib.ocm_abi_version() == declared == 2
    assert ocm.device_count() >= 0


def test_context_without_gpu_fails_loudly():
    if ocm.device_count() > 0:
        pytest.skip("a GPU is present")
    spec = synth.go_protein(20, 1)
    with pytest.raises(ocm.OCMError) as ei:
        ocm.Context(synth.build_system(spec), ocm.LangevinIntegrator(300, 0.1, 0.01, 1))
    assert ei.value.code == 2


def test_generator_size_mismatch_message():
    """Constructors reject mismatched parameter counts like the reference's
    (HarmonicBondForceFieldGenerator.hpp:30-40)."""
    with pytest.raises(ocm.OCMError) as ei:
        ocm.HarmonicBondForceFieldGenerator([[0, 1], [1, 2]], [0.38], [1.0, 1.0], False)
    assert ei.value.code == 1
    assert "HarmonicBondForceFieldGenerator: parameter number of indices_vec (2), v0 (1)" in str(ei.value)


def test_index_out_of_range_and_ionic_strength():
    sg = ocm.SystemGenerator(np.ones(3))
    sg.add_ff_generator(ocm.GoContactForceFieldGenerator([[0, 5]], [1.0], [0.5], False))
    with pytest.raises(ocm.OCMError, match="exceeds the system's largest index 2"):
        sg.generate()
    sg = ocm.SystemGenerator(np.ones(3))
    sg.add_ff_generator(ocm.DebyeHuckelForceFieldGenerator(0.0, 300, 5.5, [1, -1, 1], [], False))
    with pytest.raises(ocm.OCMError, match="ionic strength must be larger than zero"):
        sg.generate()


def test_lj_incomplete_parameter_set():
    sg = ocm.SystemGenerator(np.ones(3))
    sg.add_ff_generator(ocm.LennardJonesRepulsiveForceFieldGenerator(
        2.5, [1.0, np.nan, 1.0], [0.5, 0.5, 0.5], [], False))
    with pytest.raises(ocm.OCMError, match="should have epsilon too"):
        sg.generate()


def test_force_groups_follow_system_generator():
    spec = synth.go_protein(40, 3)
    system = synth.build_system(spec)
    assert system.group_names() == ["HarmonicBond", "GoContact", "FlexibleLocalAngle",
                                    "FlexibleLocalDihedral", "ExcludedVolume", "DebyeHuckel"]
    d = system.describe()
    fla = [f for f in d["forces"] if f["name"].startswith("FlexibleLocalAngle")]
    fld = [f for f in d["forces"] if f["name"].startswith("FlexibleLocalDihedral")]
    assert len(fla) == 20 and len(fld) == 23
    assert {f["group"] for f in fla} == {2} and {f["group"] for f in fld} == {3}


def test_derived_parameters_match_oracle():
    spec = synth.go_protein(80, 4)
    d = synth.build_system(spec).describe()
    by = {f["name"]: f for f in d["forces"]}
    r = np.sort(spec.exv.p0)[::-1]
    assert by["ExcludedVolume"]["cutoff"] == (r[0] + r[1]) * spec.exv.ratio
    assert by["ExcludedVolume"]["cutoff_correction"] == pytest.approx(
        (1.0 / by["ExcludedVolume"]["cutoff"]) ** 12, rel=1e-15)
    dh = oracle.dh_params(spec.dh.ionic_strength, spec.dh.temperature, spec.dh.ratio)
    for key, ref in (("k_e", dh["k_e"]), ("debye_length", dh["debye_length"]),
                     ("cutoff", dh["cutoff"]), ("cutoff_correction", dh["cutoff_correction"])):
        assert by["DebyeHuckel"][key] == pytest.approx(ref, rel=1e-14), key
    assert by["DebyeHuckel"]["cutoff"] == pytest.approx(2.0, rel=1e-12)
    # FLA / FLD minimum energies: the same scan as the reference, bit for bit
    for k, aa in enumerate(ocm.AMINO_ACIDS):
        assert by[f"FlexibleLocalAngle ({aa})"]["min_energy"] == oracle.fla_min_energy(k), aa
    for k, key in enumerate(ocm.fld_table_keys()):
        assert by[f"FlexibleLocalDihedral ({key})"]["min_energy"] == oracle.fld_min_energy(k), key


def test_dh_constants_at_300K_015M():
    p = oracle.dh_params(0.15, 300.0, 1.0)
    assert p["eps_r"] == pytest.approx(74.911, abs=1e-3)
    assert p["debye_length"] == pytest.approx(0.7697, abs=1e-4)
    assert p["k_e"] == pytest.approx(1.8547, abs=1e-4)


def test_lj_cutoff_and_switch():
    n = 5
    sig = np.array([0.5, 0.7, 0.6, 0.7, np.nan])
    eps = np.array([1.0, 1.0, 1.0, 1.0, np.nan])
    sg = ocm.SystemGenerator(np.ones(n))
    sg.add_ff_generator(ocm.LennardJonesRepulsiveForceFieldGenerator(2.5, eps, sig, [], False))
    sg.add_ff_generator(ocm.LennardJonesAttractiveForceFieldGenerator(2.5, eps, sig, [], False))
    d = sg.generate().describe()["forces"]
    # non-strict comparison: two equal maxima give (0.7 + 0.7) / 2 * ratio
    assert d[0]["cutoff"] == pytest.approx(0.7 * 2.5, rel=1e-15)
    assert d[1]["switch_distance"] == pytest.approx(0.9 * d[1]["cutoff"], rel=1e-15)
    assert d[0]["interaction_groups"] == 1 and d[0]["participants"] == 4


def _random_graph(rng, n):
    chain = [(i, i + 1) for i in range(n - 1)]
    extra = set()
    while len(extra) < n // 3:
        a, b = sorted(rng.integers(0, n, 2).tolist())
        if b - a > 1:
            extra.add((a, b))
    return np.array(chain), np.array(sorted(extra))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_topology_matches_oracle(seed):
    rng = np.random.default_rng(seed)
    n = 60
    bonds, contacts = _random_graph(rng, n)
    # cycles through the "bond" edges exercise the walk's visit order
    bonds = np.concatenate([bonds, contacts[:5]])
    topo = ocm.Topology(n)
    topo.add_edges(bonds, "bond")
    topo.add_edges(contacts, "contact")
    for db, dc in ((3, 1), (1, -1), (2, 2), (0, -1)):
        parts = [topo.ignore_list_within_edge(db, "bond")]
        if dc >= 0:
            parts.append(topo.ignore_list_within_edge(dc, "contact"))
        got = np.unique(np.concatenate(parts), axis=0) if sum(len(p) for p in parts) else np.zeros((0, 2))
        ref = oracle.ignore_within(n, bonds, contacts, db, dc)
        assert np.array_equal(got, ref), (db, dc)


def test_ignore_list_within_molecule():
    topo = ocm.Topology(7)
    topo.add_edges([[0, 1], [1, 2], [4, 5]], "bond")
    topo.make_molecule("bond")
    pairs = {tuple(p) for p in topo.ignore_list_within_molecule().tolist()}
    assert pairs == {(0, 1), (0, 2), (1, 2), (4, 5)}


def test_fld_class_selection_and_gly_pro_double_count():
    keys = ocm.fld_table_keys()
    aa = list(ocm.AMINO_ACIDS)
    for a1 in aa:
        for a2 in aa:
            mine = [k for k, key in enumerate(keys) if synth.fld_selects(key, a1, a2)]
            ref = oracle.fld_classes(aa.index(a1), aa.index(a2))
            assert mine == ref, (a1, a2)
    gp = oracle.fld_classes(aa.index("GLY"), aa.index("PRO"))
    assert [keys[k] for k in gp] == ["GLY-PRO", "R2-PRO"]


def test_natural_spline_matches_scipy():
    scipy_interp = pytest.importorskip("scipy.interpolate")
    y = ocm.fla_spline_table("PRO")
    h = (2.87979 - 1.30900) / 9
    M = oracle.natural_spline(y, h)
    cs = scipy_interp.CubicSpline(1.309 + h * np.arange(10), y, bc_type="natural")
    assert np.allclose(M, cs(1.309 + h * np.arange(10), 2), atol=1e-9)


def test_interaction_group_names():
    n = 6
    radii = np.full(n, 0.3)
    groups = ["A", "A", "B", "B", None, None]
    sg = ocm.SystemGenerator(np.ones(n))
    sg.add_ff_generator(ocm.ExcludedVolumeForceFieldGenerator(0.6, 2.0, radii, [], False,
                                                              ignore_group_pairs=[("A", "B")],
                                                              group_vec=groups))
    d = sg.generate().describe()["forces"][0]
    # others-others, A-others, A-A, B-others, B-B (A-B ignored)
    assert d["interaction_groups"] == 5


def test_wca_uniform_and_capped_go_generators():
    """The reference's variants: names (force groups), cutoffs, groups and
    error messages."""
    n = 6
    sig = np.array([0.5, 0.7, 0.6, 0.7, 0.4, np.nan])
    eps = np.array([1.0, 2.0, 1.0, 1.0, 0.5, np.nan])
    sg = ocm.SystemGenerator(np.ones(n))
    sg.add_ff_generator(ocm.WeeksChandlerAndersenForceFieldGenerator(sig, eps, [], False))
    sg.add_ff_generator(ocm.UniformLennardJonesAttractiveForceFieldGenerator(
        n, 0.8, 0.45, 2.5, [0, 1, 2], [3, 4, 5], [], False))
    sg.add_ff_generator(ocm.CappedGoContactForceFieldGenerator([[0, 3], [1, 4]], [1.0, 2.0], [0.6, 0.7],
                                                               0.8, False))
    system = sg.generate()
    assert system.group_names() == ["WeeksChandlerAndersen", "UniformLennardJonesAttractive",
                                    "CappedGoContact"]
    d = system.describe()["forces"]
    assert d[0]["cutoff"] == pytest.approx(2 ** (1 / 6) * 0.7, rel=1e-15)
    assert d[0]["participants"] == 5
    assert d[1]["cutoff"] == pytest.approx(0.45 * 2.5, rel=1e-15)
    assert d[1]["switch_distance"] == pytest.approx(0.9 * 0.45 * 2.5, rel=1e-15)
    assert d[1]["interaction_groups"] == 1
    # the uniform WCA keeps the reference's spelling of its name
    sg2 = ocm.SystemGenerator(np.ones(n))
    sg2.add_ff_generator(ocm.UniformWeeksChandlerAndersenForceFieldGenerator(n, 1.0, 0.5, [0, 1], [2, 3], [],
                                                                             False))
    assert sg2.generate().group_names() == ["UniformWeeksChadlerAndersen"]
    assert sg2.generate().describe()["forces"][0]["cutoff"] == pytest.approx(2 ** (1 / 6) * 0.5, rel=1e-15)
    with pytest.raises(ocm.OCMError) as ei:
        ocm.CappedGoContactForceFieldGenerator([[0, 1]], [1.0, 2.0], [0.5], 0.8, False)
    assert "CappedGoContactForceFieldGenerator : parameter number of" in str(ei.value)


def test_repulsive_slot_holds_one_generator():
    """LennardJonesRepulsive, WeeksChandlerAndersen and the uniform WCA share
    the repulsive pair slot: a second one in a system is refused."""
    n = 4
    sig, eps = np.full(n, 0.5), np.ones(n)
    sg = ocm.SystemGenerator(np.ones(n))
    sg.add_ff_generator(ocm.LennardJonesRepulsiveForceFieldGenerator(2.5, eps, sig, [], False))
    sg.add_ff_generator(ocm.WeeksChandlerAndersenForceFieldGenerator(sig, eps, [], False))
    system = sg.generate()
    # compiling the system (done by the footprint query, no GPU needed) refuses it
    assert system.footprint() == -1
    assert "share one pair slot" in ocm.lib.ocm_last_error().decode()


def _uniform_groups_ref(former, latter, ignore_pairs, group_vec):
    """Python restatement of the uniform generators' group splitting
    (UniformLennardJonesAttractiveForceFieldGenerator.cpp:28-138), empty
    sides dropped."""
    if not ignore_pairs:
        return [(set(former), set(latter))]
    related = {g for p in ignore_pairs for g in p}

    def split(side):
        named = {g: set() for g in sorted(related)}
        others = set()
        for i in side:
            g = group_vec[i]
            (named[g] if g in related else others).add(i)
        return named, others
    fn, fo = split(former)
    ln, lo = split(latter)
    out = []

    def push(a, b):
        if a and b:
            out.append((a, b))
    if fo:
        for g in ln:
            push(fo, ln[g])
        push(fo, lo)
    for fg, fs in fn.items():
        push(fs, lo)
        for lg, ls in ln.items():
            if (fg, lg) not in ignore_pairs:
                push(fs, ls)
    return out


def test_uniform_group_splitting_matches_restatement():
    n = 8
    former, latter = [0, 1, 2, 3], [4, 5, 6, 7]
    group_vec = [0, 1, 0, -1, 1, -1, 0, 1]
    ignore = [(0, 1)]
    sg = ocm.SystemGenerator(np.ones(n))
    sg.add_ff_generator(ocm.UniformLennardJonesAttractiveForceFieldGenerator(
        n, 0.5, 0.4, 2.5, former, latter, [], False, ignore_group_pairs=ignore, group_vec=group_vec))
    d = sg.generate().describe()["forces"][0]
    ref = _uniform_groups_ref(former, latter, ignore, group_vec)
    assert d["interaction_groups"] == len(ref) == 8
    # the ignored (0, 1) combination: no group pairs former-group-0 with latter-group-1
    assert ({0, 2}, {4, 7}) not in ref
