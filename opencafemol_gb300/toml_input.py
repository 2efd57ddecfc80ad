"""Reader for the part of the reference's TOML input format that the
force-and-integrate path covers.

The reference builds its OpenMM System from one TOML file
(src/input/ReadTOMLInput.cpp:20-875, src/input/ReadTOMLForceFieldGenerator.cpp).
This module reads the same file layout into a ``synth.CGSpec`` (the flat
description the engines and the generators consume), with the reader's unit
conversions:

* positions and lengths: Angstrom -> nm (``pos``, ``v0``, ``radius``,
  ``sigma``, box lengths: ReadTOMLInput.cpp:71-73, 920-923);
* energies: kcal/mol -> kJ/mol (``k`` of GoContact, FLA and FLD, ``epsilon``);
* harmonic bonds: the file's ``k (r - v0)^2`` becomes OpenMM's
  ``1/2 k' (r - v0)^2`` with ``k' = 2 k * 4.184 * 100``
  (ReadTOMLForceFieldGenerator.cpp:57-64);
* velocities: Angstrom / cafetime -> nm/ps, ``delta_t`` in cafetime,
  ``gamma_t`` (default 0.01) in 1/cafetime (ReadTOMLInput.cpp:876-905,
  930-960), cafetime = sqrt(1/4.184) * 0.1 ps (src/util/Constants.hpp:23);
* cutoffs of the pair terms are ratios with the reader's defaults:
  ExcludedVolume 2.0, DebyeHuckel 5.5, Lennard-Jones 2.5
  (ReadTOMLForceFieldGenerator.cpp:1080, 1381, 2126-2127, 2194-2195);
* ``ignore.particles_within`` tables become exclusions within that many
  edges of the named type (ReadTOMLForceFieldGenerator.cpp:963-1013);
* FlexibleLocalAngle parameters are selected per residue by the ``y``
  name ("y1_PHE" -> PHE) and FlexibleLocalDihedral parameters by the
  ``coef`` pair, with the reader's GLY/PRO rules (including a GLY-PRO coef
  counted by both the GLY-PRO and the R2-PRO class).

* AICG2+ Gaussian bonds (k kcal/mol -> kJ/mol, v0 and sigma Angstrom -> nm)
  and Gaussian dihedrals (k kcal/mol -> kJ/mol, v0 and sigma in radians)
  (ReadTOMLForceFieldGenerator.cpp:92-150, 494-540).

Terms outside the covered set (cosine dihedrals, 3SPN2, WCA, walls,
group-based ignores, molecule-based ignores) raise ``ValueError``, or, with
``strict=False``, are left out and listed in ``skipped``.
"""
from __future__ import annotations

import math
import tomllib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .forcefield import AMINO_ACIDS, LangevinIntegratorGenerator
from .synth import CGSpec, PairTerm

KJ_PER_KCAL = 4.184
NM_PER_ANGSTROM = 0.1
CAFETIME_PS = math.sqrt(1.0 / KJ_PER_KCAL) * 0.1

_PAIR_DEFAULT_RATIO = {"ExcludedVolume": 2.0, "DebyeHuckel": 5.5,
                       "LennardJonesRepulsive": 2.5, "LennardJonesAttractive": 2.5,
                       "WCA": 0.0}  # the WCA cutoff is 2^(1/6) sigma, no ratio


@dataclass
class TomlSystem:
    spec: CGSpec
    integrator: LangevinIntegratorGenerator
    velocities: np.ndarray | None          # nm/ps, None when the file has none
    total_step: int = 0
    save_step: int = 0
    energy_minimization: bool = False      # [simulator] energy_minimization (ReadTOMLInput.cpp:1008)
    seed: int = 0
    group_vec: list = field(default_factory=list)
    skipped: list = field(default_factory=list)


def _aa_index(name: str) -> int:
    try:
        return AMINO_ACIDS.index(name)
    except ValueError:
        raise ValueError(f"unknown residue name {name!r}") from None


class _Params(dict):
    """One parameter table with the block's `env` table: a value written as
    a string names an entry of `env` (Utility.hpp find_parameter, :33-139).
    The table-name keys (y, d2y, coef, name) are plain strings."""

    _NAMES = ("y", "d2y", "coef", "name")

    def __init__(self, p: dict, env: dict | None):
        super().__init__(p)
        self.env = env or {}

    def __getitem__(self, key):
        v = super().__getitem__(key)
        if isinstance(v, str) and key not in self._NAMES:
            if not self.env:
                raise ValueError(f'named variable "{v}" used but no env is defined')
            if v not in self.env:
                raise ValueError(f'named variable "{v}" used but not defined in env')
            v = self.env[v]
        return v

    def get(self, key, default=None):
        return self[key] if key in self else default

    def get_or(self, key, default):
        """Lenient lookup of an optional key (Utility.hpp find_parameter_or,
        :140-155): a missing key, or a name that env does not define, gives
        the default instead of an error."""
        if key not in self:
            return default
        v = super().__getitem__(key)
        if isinstance(v, str):
            return self.env.get(v, default)
        return v


def _params(block: dict):
    env = block.get("env")
    return [_Params(p, env) for p in block["parameters"]]


def _offset(p: dict) -> int:
    """The optional index offset, read as the reference reads it
    (find_parameter_or(params, env, "offset", 0))."""
    return int(p.get_or("offset", 0) if isinstance(p, _Params) else p.get("offset", 0))


def _index(p: dict) -> int:
    return int(p["index"]) + _offset(p)


def _indices(p: dict) -> list[int]:
    off = _offset(p)
    return [int(v) + off for v in p["indices"]]


def _check_range(idx, n: int, what: str) -> None:
    for v in np.atleast_1d(idx):
        if v < 0 or v >= n:
            raise ValueError(f"[error] {what} : index {int(v)} exceeds the system's largest index {n - 1}.")


def _ignore_groups(ff: dict) -> list[tuple[str, str]]:
    """ignore.group.inter = [[A, B], ...] and ignore.group.intra = [A, ...]
    (ReadTOMLForceFieldGenerator.cpp:1016-1050) as (name, name) pairs."""
    grp = ff.get("ignore", {}).get("group", {})
    pairs = [(str(a), str(b)) for a, b in grp.get("inter", [])]
    pairs += [(str(a), str(a)) for a in grp.get("intra", [])]
    return pairs


def _ignore_molecule(ff: dict) -> bool:
    """ignore.molecule = "Intra" / "Self": no pair inside one bond-connected
    molecule (ReadTOMLForceFieldGenerator.cpp:963-985)."""
    return ff.get("ignore", {}).get("molecule", "Nothing") in ("Intra", "Self")


def _ignore_within(ff: dict, what: str) -> tuple[int, int]:
    ign = ff.get("ignore", {})
    mol = ign.get("molecule", "Nothing")
    if mol in ("Others", "Inter"):
        raise ValueError('[error] ignore molecule do not support "Others" or "Inter".')
    within = ign.get("particles_within", {})
    unknown = set(within) - {"bond", "contact"}
    if unknown:
        raise ValueError(f"{what}: particles_within over {sorted(unknown)} is not supported")
    return int(within.get("bond", -1)), int(within.get("contact", -1))


def _per_particle(ff: dict, n: int, keys: tuple[str, ...], what: str) -> list[np.ndarray]:
    out = [np.full(n, np.nan) for _ in keys]
    for p in _params(ff):
        i = _index(p)
        _check_range(i, n, what)
        for arr, k in zip(out, keys):
            arr[i] = float(p[k])
    return out


def _either(p: dict, a: str, b: str):
    return p[a] if a in p else p[b]


def _uniform_table(glob: dict, n: int, what: str):
    """The one (sigma nm, epsilon kJ/mol, side bits) of a uniform-form type
    table ([forcefields.global.table.A.B]); former = particles named A,
    latter = particles named B (ReadTOMLInput.cpp:435-512, 546-621,
    ReadTOMLForceFieldGenerator.cpp:1307-1357).  Pairs with an empty side are
    skipped, as in the reference; more than one remaining pair type would
    need one pair slot each and is reported as not covered."""
    names = {}
    for p in _params(glob):
        i = _index(p)
        _check_range(i, n, "read_toml_uniform_ff_generator")
        names.setdefault(str(p["name"]), []).append(i)
    found = []
    for first, sub in glob["table"].items():
        for second, par in sub.items():
            former, latter = names.get(first, []), names.get(second, [])
            if not former or not latter:
                continue
            side = np.zeros(n, np.int8)
            side[former] |= 1
            side[latter] |= 2
            found.append((float(_either(par, "sigma", "σ")) * NM_PER_ANGSTROM,
                          float(_either(par, "epsilon", "ε")) * KJ_PER_KCAL, side))
    if len(found) != 1:
        raise ValueError(f"{what}: a type table with {len(found)} interacting pair types "
                         "(one is covered: each needs its own pair slot)")
    return found[0]


def read_toml(source, strict: bool = True, fp32_positions: bool = True) -> TomlSystem:
    """Read a reference input file (path, bytes or an already-parsed dict).

    With ``fp32_positions`` the coordinates are rounded to FP32-representable
    values (periodic ones after wrapping into the box, whose lengths are
    rounded to FP32 too), so the FP64 oracle and
    the FP32 kernels see the same input."""
    if isinstance(source, dict):
        data = source
    elif isinstance(source, (bytes, bytearray)):
        data = tomllib.loads(source.decode())
    else:
        with open(Path(source), "rb") as fh:
            data = tomllib.load(fh)
    skipped: list[str] = []

    def unsupported(msg: str) -> None:
        if strict:
            raise ValueError(msg)
        skipped.append(msg)

    system = data["systems"][0]
    particles = system["particles"]
    n = len(particles)
    masses = np.array([float(p["m"] if "m" in p else p["mass"]) for p in particles])
    pos = np.array([p["pos"] if "pos" in p else p["position"] for p in particles], float) * NM_PER_ANGSTROM
    vel = None
    if "vel" in particles[0] or "velocity" in particles[0]:
        vel = np.array([p["vel"] if "vel" in p else p["velocity"] for p in particles], float)
        vel *= NM_PER_ANGSTROM / CAFETIME_PS
    group_vec = [p.get("group") for p in particles]
    attr = system.get("attributes", {})
    sim = data["simulator"]
    temperature = float(attr["temperature"])
    dt = float(sim["delta_t"]) * CAFETIME_PS
    friction = float(sim.get("gamma_t", 0.01)) / CAFETIME_PS
    seed = int(sim.get("seed", 0))

    periodic = sim["boundary_type"] in ("Periodic", "PeriodicCuboid")
    box = None
    if periodic:
        shape = system["boundary_shape"]
        box = tuple((float(u) - float(lo)) * NM_PER_ANGSTROM for lo, u in zip(shape["lower"], shape["upper"]))
    elif sim["boundary_type"] != "Unlimited":
        raise ValueError(f"unknown boundary_type {sim['boundary_type']!r}")
    if fp32_positions:
        if periodic:
            # the kernels hold the box and the wrapped coordinates in FP32:
            # rounding the box and wrapping before rounding the coordinates
            # makes these the values they use
            box = tuple(float(np.float32(b)) for b in box)
            L = np.array(box)
            pos = pos - L * np.floor(pos / L)
        pos = pos.astype(np.float32).astype(np.float64)
        if periodic:
            pos = np.where(pos >= L, pos - L, pos)

    spec = CGSpec(n=n, pos=pos, masses=masses, periodic=periodic, box=box, temperature=temperature,
                  friction=friction, dt=dt)
    bonds, bond_v0, bond_k = [], [], []
    contacts, go_k, go_r0 = [], [], []
    fla_idx, fla_k, fla_aa = [], [], []
    fld_idx, fld_k, fld_aa1, fld_aa2 = [], [], [], []
    gb_idx, gb_k, gb_v0, gb_sigma = [], [], [], []
    gd_idx, gd_k, gd_theta0, gd_sigma = [], [], [], []
    cgo_idx, cgo_k, cgo_r0, cgo_cap = [], [], [], []
    cgo_topology = None
    ff = data["forcefields"][0]
    for loc in ff.get("local", []):
        inter, pot = loc["interaction"], loc["potential"]
        what = f"{inter}/{pot}"
        if inter == "BondLength" and pot == "Harmonic":
            for p in _params(loc):
                ij = _indices(p)
                _check_range(ij, n, "read_toml_harmonic_bond_ff_generator")
                bonds.append(ij)
                bond_v0.append(float(p["v0"]) * NM_PER_ANGSTROM)
                bond_k.append(float(p["k"]) * KJ_PER_KCAL * 100.0 * 2.0)
            if loc.get("topology") != "bond":
                unsupported(f"{what}: only topology = \"bond\" is covered")
        elif inter == "BondLength" and pot == "GoContact":
            for p in _params(loc):
                ij = _indices(p)
                _check_range(ij, n, "read_toml_go_contact_ff_generator")
                contacts.append(ij)
                go_k.append(float(p["k"]) * KJ_PER_KCAL)
                go_r0.append(float(p["v0"]) * NM_PER_ANGSTROM)
            if loc.get("topology") != "contact":
                unsupported(f"{what}: only topology = \"contact\" is covered")
        elif inter == "BondLength" and pot == "CappedGoContact":
            cap = float(loc.get("capping_ratio", 0.75))  # ReadTOMLForceFieldGenerator.cpp:237
            for p in _params(loc):
                ij = _indices(p)
                _check_range(ij, n, "read_toml_capped_go_contact_ff_generator")
                cgo_idx.append(ij)
                cgo_k.append(float(p["k"]) * KJ_PER_KCAL)
                cgo_r0.append(float(p["v0"]) * NM_PER_ANGSTROM)
                cgo_cap.append(cap)
            topo = loc.get("topology", "none")
            if topo not in ("none", "contact") or (cgo_topology is not None and topo != cgo_topology):
                unsupported(f"{what}: only one topology (\"none\" or \"contact\") for all blocks is covered")
            cgo_topology = topo
        elif inter == "BondLength" and pot == "Gaussian":
            for p in _params(loc):
                ij = _indices(p)
                _check_range(ij, n, "read_toml_gaussian_bond_ff_generator")
                gb_idx.append(ij)
                gb_k.append(float(p["k"]) * KJ_PER_KCAL)
                gb_v0.append(float(p["v0"]) * NM_PER_ANGSTROM)
                gb_sigma.append(float(p["sigma"] if "sigma" in p else p["σ"]) * NM_PER_ANGSTROM)
            if loc.get("topology", "none") != "none":
                unsupported(f"{what}: only topology = \"none\" is covered")
        elif inter == "DihedralAngle" and pot == "Gaussian":
            for p in _params(loc):
                ijkl = _indices(p)
                _check_range(ijkl, n, "read_toml_gaussian_dihedral_ff_generator")
                gd_idx.append(ijkl)
                gd_k.append(float(p["k"]) * KJ_PER_KCAL)
                gd_theta0.append(float(p["v0"]))  # radian
                gd_sigma.append(float(p["sigma"] if "sigma" in p else p["σ"]))  # radian
            if loc.get("topology", "none") != "none":
                unsupported(f"{what}: only topology = \"none\" is covered")
        elif inter == "BondAngle" and pot == "FlexibleLocalAngle":
            for p in _params(loc):
                ijk = _indices(p)
                _check_range(ijk, n, "read_toml_flexible_local_angle_ff_generator")
                fla_idx.append(ijk)
                fla_k.append(float(p["k"]) * KJ_PER_KCAL)
                fla_aa.append(_aa_index(str(p["y"])[3:6]))
        elif inter == "DihedralAngle" and pot == "FlexibleLocalDihedral":
            for p in _params(loc):
                ijkl = _indices(p)
                _check_range(ijkl, n, "read_toml_flexible_local_dihedral_ff_generator")
                coef = str(p["coef"])
                fld_idx.append(ijkl)
                fld_k.append(float(p["k"]) * KJ_PER_KCAL)
                fld_aa1.append(_aa_index(coef[0:3]))
                fld_aa2.append(_aa_index(coef[4:7]))
        else:
            unsupported(f"local force {what} is not covered")
    if bonds:
        spec.bonds = np.array(bonds, np.int64)
        spec.bond_v0, spec.bond_k = np.array(bond_v0), np.array(bond_k)
    if contacts:
        spec.contacts = np.array(contacts, np.int64)
        spec.go_k, spec.go_r0 = np.array(go_k), np.array(go_r0)
    if gb_idx:
        spec.gb_idx, spec.gb_k = np.array(gb_idx, np.int64), np.array(gb_k)
        spec.gb_v0, spec.gb_sigma = np.array(gb_v0), np.array(gb_sigma)
    if gd_idx:
        spec.gd_idx, spec.gd_k = np.array(gd_idx, np.int64), np.array(gd_k)
        spec.gd_theta0, spec.gd_sigma = np.array(gd_theta0), np.array(gd_sigma)
    if fla_idx:
        spec.fla_idx, spec.fla_k = np.array(fla_idx, np.int64), np.array(fla_k)
        spec.fla_aa = np.array(fla_aa, np.int32)
    if fld_idx:
        spec.fld_idx, spec.fld_k = np.array(fld_idx, np.int64), np.array(fld_k)
        spec.fld_aa1, spec.fld_aa2 = np.array(fld_aa1, np.int32), np.array(fld_aa2, np.int32)
    if cgo_idx:
        spec.cgo_idx, spec.cgo_k, spec.cgo_r0 = np.array(cgo_idx, np.int64), np.array(cgo_k), np.array(cgo_r0)
        spec.cgo_cap = np.array(cgo_cap)
        spec.cgo_topology = cgo_topology or "none"

    for glob in ff.get("global", []):
        pot = glob["potential"]
        what = f"{glob.get('interaction', 'Pair')}/{pot}"
        if pot not in _PAIR_DEFAULT_RATIO:
            unsupported(f"global force {what} is not covered")
            continue
        if "table" in glob and pot not in ("WCA", "LennardJonesAttractive"):
            unsupported(f"global force {what} with a type table (uniform form) is not covered")
            continue
        try:
            ign_bond, ign_contact = _ignore_within(glob, what)
        except ValueError as e:
            unsupported(str(e))
            continue
        ratio = float(glob.get("cutoff", _PAIR_DEFAULT_RATIO[pot]))
        ign_groups = _ignore_groups(glob) or None
        ign_mol = _ignore_molecule(glob)
        if ign_groups:
            spec.group_names = list(group_vec)
        if "table" in glob:  # uniform WCA / uniform attractive LJ between two named particle sets
            try:
                sig, eps, side = _uniform_table(glob, n, what)
            except ValueError as e:
                unsupported(str(e))
                continue
            t = PairTerm(ratio=ratio, p0=np.full(n, eps), p1=np.full(n, sig), kind="uniform", side=side,
                         ign_bond=ign_bond, ign_contact=ign_contact, ignore_groups=ign_groups, ign_molecule=ign_mol)
            if pot == "WCA":
                spec.ljr = t
            else:
                spec.lja = t
            continue
        if pot == "ExcludedVolume":
            (radius,) = _per_particle(glob, n, ("radius",), "read_toml_excluded_volume_ff_generator")
            spec.exv = PairTerm(ratio=ratio, p0=radius * NM_PER_ANGSTROM,
                                eps=float(glob["epsilon"]) * KJ_PER_KCAL, ign_bond=ign_bond,
                                ign_contact=ign_contact, ignore_groups=ign_groups, ign_molecule=ign_mol)
        elif pot == "DebyeHuckel":
            (q,) = _per_particle(glob, n, ("charge",), "read_toml_debye_huckel_ff_generator")
            if "ionic_strength" not in attr:
                raise ValueError("[error] attributes table must contains ionic_strength for DebyeHuckel potential.")
            spec.dh = PairTerm(ratio=ratio, p0=q, ionic_strength=float(attr["ionic_strength"]),
                               temperature=temperature, ign_bond=ign_bond, ign_contact=ign_contact,
                               ignore_groups=ign_groups, ign_molecule=ign_mol)
        elif pot == "WCA":
            sig, eps = np.full(n, np.nan), np.full(n, np.nan)
            for p in _params(glob):
                i = _index(p)
                _check_range(i, n, "read_toml_weeks_chandler_andersen_ff_generator")
                sig[i] = float(_either(p, "sigma", "σ"))
                eps[i] = float(_either(p, "epsilon", "ε"))
            spec.ljr = PairTerm(ratio=0.0, p0=eps * KJ_PER_KCAL, p1=sig * NM_PER_ANGSTROM, kind="wca",
                                ign_bond=ign_bond, ign_contact=ign_contact, ignore_groups=ign_groups, ign_molecule=ign_mol)
        else:
            eps, sig = _per_particle(glob, n, ("epsilon", "sigma"),
                                     "read_toml_lennard_jones_ff_generator")
            t = PairTerm(ratio=ratio, p0=eps * KJ_PER_KCAL, p1=sig * NM_PER_ANGSTROM, ign_bond=ign_bond,
                         ign_contact=ign_contact, ignore_groups=ign_groups, ign_molecule=ign_mol)
            if pot == "LennardJonesRepulsive":
                spec.ljr = t
            else:
                spec.lja = t

    integ = LangevinIntegratorGenerator(temperature, friction, dt, seed)
    return TomlSystem(spec=spec, integrator=integ, velocities=vel,
                      total_step=int(sim.get("total_step", 0)), save_step=int(sim.get("save_step", 0)),
                      energy_minimization=bool(sim.get("energy_minimization", False)),
                      seed=seed, group_vec=group_vec, skipped=skipped)
