"""Host-side mirror of the reference's force-field generators, topology and
system assembly, bound to the C ABI.

Class names, constructor arguments and their meaning follow the reference
(src/forcefield/*ForceFieldGenerator.hpp, src/Topology.hpp,
src/SystemGenerator.hpp, src/IntegratorGenerator.hpp).  Units are OpenMM's
(nm, kJ/mol, amu, ps): the unit conversions of the TOML readers are applied
by the caller, as in the reference.  ``std::nullopt`` per-particle values are
``NaN`` here.  Errors raise ``OCMError`` carrying the engine's message.
"""
from __future__ import annotations

import ctypes as C
import json
import math
from typing import Sequence

import numpy as np

from ._lib import (OCMError, as_f64, as_i32, as_i64, check, dptr, i32ptr, i64ptr, lib)

__all__ = [
    "Topology", "HarmonicBondForceFieldGenerator", "GoContactForceFieldGenerator",
    "GaussianBondForceFieldGenerator", "GaussianDihedralForceFieldGenerator",
    "FlexibleLocalAngleForceFieldGenerator", "FlexibleLocalDihedralForceFieldGenerator",
    "ExcludedVolumeForceFieldGenerator", "DebyeHuckelForceFieldGenerator",
    "LennardJonesRepulsiveForceFieldGenerator", "LennardJonesAttractiveForceFieldGenerator",
    "WeeksChandlerAndersenForceFieldGenerator", "UniformWeeksChandlerAndersenForceFieldGenerator",
    "UniformLennardJonesAttractiveForceFieldGenerator", "CappedGoContactForceFieldGenerator",
    "SystemGenerator", "System", "LangevinIntegratorGenerator", "LangevinIntegrator",
    "fla_spline_table", "fla_second_derivative_table", "fld_fourier_table", "fld_table_keys",
    "AMINO_ACIDS",
]

AMINO_ACIDS = ("ALA", "ARG", "ASN", "ASP", "CYS", "GLN", "GLU", "GLY", "HIS", "ILE",
               "LEU", "LYS", "MET", "PHE", "PRO", "SER", "THR", "TRP", "TYR", "VAL")


def fla_spline_table(aa: str) -> np.ndarray:
    y = np.zeros(10)
    check(lib.ocm_fla_table(aa.encode(), dptr(y), None))
    return y


def fla_second_derivative_table(aa: str) -> np.ndarray:
    d = np.zeros(10)
    check(lib.ocm_fla_table(aa.encode(), None, dptr(d)))
    return d


def fld_fourier_table(key: str) -> np.ndarray:
    f = np.zeros(7)
    check(lib.ocm_fld_table(key.encode(), dptr(f)))
    return f


def fld_table_keys() -> list[str]:
    out = []
    buf = C.create_string_buffer(32)
    for k in range(23):
        check(lib.ocm_fld_table_key(k, buf, 32))
        out.append(buf.value.decode())
    return out


# ---------------------------------------------------------------------------
class Topology:
    """Bond / contact graph (src/Topology.hpp:9-81)."""

    def __init__(self, system_size: int):
        h = C.c_void_p()
        check(lib.ocm_topology_create(int(system_size), C.byref(h)))
        self._h = h
        self._n = int(system_size)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.ocm_topology_destroy(h)
            self._h = None

    def size(self) -> int:
        return self._n

    def add_edges(self, edges, edge_type: str) -> None:
        e = as_i64(edges).reshape(-1, 2) if len(edges) else np.zeros((0, 2), np.int64)
        check(lib.ocm_topology_add_edges(self._h, len(e), i64ptr(e), edge_type.encode()))

    def make_molecule(self, edge_type: str) -> None:
        check(lib.ocm_topology_make_molecule(self._h, edge_type.encode()))

    def _pairs(self, fn, *args) -> np.ndarray:
        n = C.c_int64()
        cap = 1024
        while True:
            out = np.zeros((cap, 2), np.int64)
            code = fn(self._h, *args, i64ptr(out), cap, C.byref(n))
            if code == 0:
                return out[: n.value].copy()
            if n.value > cap:
                cap = n.value
                continue
            check(code)

    def ignore_list_within_edge(self, dist: int, edge_type: str) -> np.ndarray:
        return self._pairs(lib.ocm_topology_ignore_list_within_edge, int(dist), edge_type.encode())

    def ignore_list_within_molecule(self) -> np.ndarray:
        return self._pairs(lib.ocm_topology_ignore_list_within_molecule)


# ---------------------------------------------------------------------------
class _Generator:
    def add_to(self, sys_handle) -> int:  # pragma: no cover - overridden
        raise NotImplementedError


def _pairs_arg(indices, width: int) -> np.ndarray:
    arr = as_i64(indices)
    if arr.size == 0:
        return np.zeros((0, width), np.int64)
    return arr.reshape(-1, width)


class HarmonicBondForceFieldGenerator(_Generator):
    """1/2 k (r - v0)^2; ``ks`` are already doubled by the reader."""

    def __init__(self, indices_vec, v0s, ks, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 2)
        self.v0s, self.ks = as_f64(v0s), as_f64(ks)
        self.use_periodic = bool(use_periodic)
        if not (len(self.indices) == len(self.v0s) == len(self.ks)):
            raise OCMError(1, "[error] HarmonicBondForceFieldGenerator: parameter number of "
                              f"indices_vec ({len(self.indices)}), v0 ({len(self.v0s)}) and "
                              f"k ({len(self.ks)}) is not matched.The number os these parameters must be same.")

    def name(self) -> str:
        return "HarmonicBond"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_harmonic_bond(h, len(self.indices), i64ptr(self.indices), dptr(self.v0s),
                                        dptr(self.ks), int(self.use_periodic), C.byref(g)))
        return g.value


class GoContactForceFieldGenerator(_Generator):
    """k (5 (r0/r)^12 - 6 (r0/r)^10)."""

    def __init__(self, indices_vec, ks, r0s, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 2)
        self.ks, self.r0s = as_f64(ks), as_f64(r0s)
        self.use_periodic = bool(use_periodic)
        if not (len(self.indices) == len(self.ks) == len(self.r0s)):
            raise OCMError(1, "[error] GoContactForceFieldGenerator : parameter number of "
                              f"indices_vec ({len(self.indices)}), k ({len(self.ks)}) and "
                              f"r0 ({len(self.r0s)}) is not matched.The number of these parameters must be same.")

    def name(self) -> str:
        return "GoContact"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_go_contact(h, len(self.indices), i64ptr(self.indices), dptr(self.ks),
                                     dptr(self.r0s), int(self.use_periodic), C.byref(g)))
        return g.value


class GaussianBondForceFieldGenerator(_Generator):
    """AICG2+ k exp(-(r - v0)^2 / (2 sigma^2)); ks in kJ/mol, v0s and sigmas in nm."""

    def __init__(self, indices_vec, ks, v0s, sigmas, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 2)
        self.ks, self.v0s, self.sigmas = as_f64(ks), as_f64(v0s), as_f64(sigmas)
        self.use_periodic = bool(use_periodic)
        if not (len(self.indices) == len(self.ks) == len(self.v0s) == len(self.sigmas)):
            raise OCMError(1, "[error] GaussianBondForceFieldGenerator: parameter number of "
                              f"indices_vec ({len(self.indices)}), k ({len(self.ks)}), v0 ({len(self.v0s)}) "
                              f"and sigmas ({len(self.sigmas)}) is not matched."
                              "The number of these parameters must be same.")

    def name(self) -> str:
        return "GaussianBond"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_gaussian_bond(h, len(self.indices), i64ptr(self.indices), dptr(self.ks),
                                        dptr(self.v0s), dptr(self.sigmas), int(self.use_periodic),
                                        C.byref(g)))
        return g.value


class GaussianDihedralForceFieldGenerator(_Generator):
    """AICG2+ k exp(-dphi^2 / (2 sigma^2)), dphi = phi - theta0 wrapped to
    [-pi, pi); theta0s and sigmas in radians."""

    def __init__(self, indices_vec, ks, theta0s, sigmas, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 4)
        self.ks, self.theta0s, self.sigmas = as_f64(ks), as_f64(theta0s), as_f64(sigmas)
        self.use_periodic = bool(use_periodic)
        if not (len(self.indices) == len(self.ks) == len(self.theta0s) == len(self.sigmas)):
            raise OCMError(1, "[error] GaussianDihedralForceFieldGenerator : parameter number of "
                              f"indices_vec ({len(self.indices)}), k ({len(self.ks)}), theta0 "
                              f"({len(self.theta0s)}) and simga ({len(self.sigmas)} is not matched."
                              "The number of these parameters must be same.")

    def name(self) -> str:
        return "GaussianDihedral"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_gaussian_dihedral(h, len(self.indices), i64ptr(self.indices), dptr(self.ks),
                                            dptr(self.theta0s), dptr(self.sigmas), int(self.use_periodic),
                                            C.byref(g)))
        return g.value


class FlexibleLocalAngleForceFieldGenerator(_Generator):
    def __init__(self, indices_vec, ks, spline_table, aa_name: str, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 3)
        self.ks = as_f64(ks)
        self.table = as_f64(spline_table)
        if self.table.shape != (10,):
            raise OCMError(1, "spline_table must have 10 values")
        self.aa = aa_name
        self.use_periodic = bool(use_periodic)
        if len(self.indices) != len(self.ks):
            raise OCMError(1, "[error] FlexibleLocalAngleForceFieldGenerator : parameter number of"
                              f"indices_vec ({len(self.indices)}) and k ({len(self.ks)}) is not matched."
                              "The number of these parameters must be same.")

    def name(self) -> str:
        return f"FlexibleLocalAngle ({self.aa})"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_flexible_local_angle(h, len(self.indices), i64ptr(self.indices), dptr(self.ks),
                                               dptr(self.table), self.aa.encode(),
                                               int(self.use_periodic), C.byref(g)))
        return g.value


class FlexibleLocalDihedralForceFieldGenerator(_Generator):
    def __init__(self, indices_vec, ks, fourier_table, aa_pair_name: str, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 4)
        self.ks = as_f64(ks)
        self.table = as_f64(fourier_table)
        if self.table.shape != (7,):
            raise OCMError(1, "fourier_table must have 7 values")
        self.pair = aa_pair_name
        self.use_periodic = bool(use_periodic)
        if len(self.indices) != len(self.ks):
            raise OCMError(1, "[error] FlexibleLocalDihedralForceFieldGenerator : parameter number of "
                              f"indices_vec ({len(self.indices)}) and k ({len(self.ks)}) is not matched."
                              "The number of these parameters must be same.")

    def name(self) -> str:
        return f"FlexibleLocalDihedral ({self.pair})"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_flexible_local_dihedral(h, len(self.indices), i64ptr(self.indices),
                                                  dptr(self.ks), dptr(self.table), self.pair.encode(),
                                                  int(self.use_periodic), C.byref(g)))
        return g.value


def _group_args(ignore_group_pairs, group_vec, n: int):
    """Map group names to ids in lexicographic order; -1 = no group."""
    if not ignore_group_pairs:
        return 0, None, None
    names = sorted({g for g in group_vec if g is not None} | {a for p in ignore_group_pairs for a in p})
    ids = {nm: k for k, nm in enumerate(names)}
    igp = as_i32([ids[a] for p in ignore_group_pairs for a in p])
    gv = as_i32([ids[g] if g is not None else -1 for g in group_vec])
    if len(gv) != n:
        raise OCMError(1, "group_vec must have one entry per particle")
    return len(ignore_group_pairs), igp, gv


class _PairGenerator(_Generator):
    def _common(self, ignore_list, use_periodic, ignore_group_pairs, group_vec):
        self.ignore = _pairs_arg(ignore_list, 2) if ignore_list is not None else np.zeros((0, 2), np.int64)
        self.use_periodic = bool(use_periodic)
        self.ignore_group_pairs = list(ignore_group_pairs or [])
        self.group_vec = list(group_vec or [])

    def _tail(self, n: int):
        ng, igp, gv = _group_args(self.ignore_group_pairs, self.group_vec, n)
        return (len(self.ignore), i64ptr(self.ignore), int(self.use_periodic), ng, i32ptr(igp), i32ptr(gv))


class ExcludedVolumeForceFieldGenerator(_PairGenerator):
    """eps (s_i + s_j)^12 (r^-12 - rc^-12), rc = cutoff * (max + 2nd max radius)."""

    def __init__(self, eps: float, cutoff: float, radii, ignore_list, use_periodic: bool,
                 ignore_group_pairs=(), group_vec=()):
        self.eps, self.cutoff = float(eps), float(cutoff)
        self.radii = as_f64(radii)
        self._common(ignore_list, use_periodic, ignore_group_pairs, group_vec)

    def name(self) -> str:
        return "ExcludedVolume"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_excluded_volume(h, self.eps, self.cutoff, dptr(self.radii),
                                          *self._tail(len(self.radii)), C.byref(g)))
        return g.value


class DebyeHuckelForceFieldGenerator(_PairGenerator):
    def __init__(self, ionic_strength: float, temperature: float, cutoff_ratio: float, charges,
                 ignore_list, use_periodic: bool, ignore_group_pairs=(), group_vec=()):
        self.ionic_strength, self.temperature = float(ionic_strength), float(temperature)
        self.cutoff_ratio = float(cutoff_ratio)
        self.charges = as_f64(charges)
        self._common(ignore_list, use_periodic, ignore_group_pairs, group_vec)

    def name(self) -> str:
        return "DebyeHuckel"

    @staticmethod
    def dielectric_water(T: float, C_: float) -> float:
        return (249.4 - 0.788 * T + 7.2e-4 * T * T) * (1. - 2.551e-1 * C_ + 5.151e-2 * C_ * C_
                                                       - 6.889e-3 * C_ * C_ * C_)

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_debye_huckel(h, self.ionic_strength, self.temperature, self.cutoff_ratio,
                                       dptr(self.charges), *self._tail(len(self.charges)), C.byref(g)))
        return g.value


class LennardJonesRepulsiveForceFieldGenerator(_PairGenerator):
    def __init__(self, cutoff_ratio: float, epsilons, sigmas, ignore_list, use_periodic: bool,
                 ignore_group_pairs=(), group_vec=()):
        self.cutoff_ratio = float(cutoff_ratio)
        self.epsilons, self.sigmas = as_f64(epsilons), as_f64(sigmas)
        self._common(ignore_list, use_periodic, ignore_group_pairs, group_vec)

    def name(self) -> str:
        return "LennardJonesRepulsive"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_lennard_jones_repulsive(h, self.cutoff_ratio, dptr(self.epsilons),
                                                  dptr(self.sigmas), *self._tail(len(self.sigmas)),
                                                  C.byref(g)))
        return g.value


class LennardJonesAttractiveForceFieldGenerator(LennardJonesRepulsiveForceFieldGenerator):
    def name(self) -> str:
        return "LennardJonesAttractive"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_lennard_jones_attractive(h, self.cutoff_ratio, dptr(self.epsilons),
                                                   dptr(self.sigmas), *self._tail(len(self.sigmas)),
                                                   C.byref(g)))
        return g.value


class WeeksChandlerAndersenForceFieldGenerator(_PairGenerator):
    """step(2^(1/6) s - r) (4 e ((s/r)^12 - (s/r)^6) + e); s arithmetic, e
    geometric mean; cutoff 2^(1/6) (s_max + s_2nd) / 2."""

    def __init__(self, sigmas, epsilons, ignore_list, use_periodic: bool, ignore_group_pairs=(), group_vec=()):
        self.sigmas, self.epsilons = as_f64(sigmas), as_f64(epsilons)
        if len(self.sigmas) != len(self.epsilons):
            raise OCMError(1, f"WCA: sigma.size(={len(self.sigmas)}) must be the same as "
                              f"epsilon.size(={len(self.epsilons)})")
        self._common(ignore_list, use_periodic, ignore_group_pairs, group_vec)

    def name(self) -> str:
        return "WeeksChandlerAndersen"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_weeks_chandler_andersen(h, dptr(self.sigmas), dptr(self.epsilons),
                                                  *self._tail(len(self.sigmas)), C.byref(g)))
        return g.value


class _UniformPairGenerator(_PairGenerator):
    def _uniform(self, system_size, eps, sigma, former_group_vec, latter_group_vec):
        self.system_size = int(system_size)
        self.eps, self.sigma = float(eps), float(sigma)
        self.former = np.ascontiguousarray(former_group_vec, np.int64).reshape(-1)
        self.latter = np.ascontiguousarray(latter_group_vec, np.int64).reshape(-1)


class UniformWeeksChandlerAndersenForceFieldGenerator(_UniformPairGenerator):
    """4 eps ((sigma/r)^12 - (sigma/r)^6 + 1/4) between `former` and `latter`,
    cutoff 2^(1/6) sigma."""

    def __init__(self, system_size, eps, sigma, former_group_vec, latter_group_vec, ignore_list,
                 use_periodic: bool, ignore_group_pairs=(), group_vec=()):
        self._uniform(system_size, eps, sigma, former_group_vec, latter_group_vec)
        self._common(ignore_list, use_periodic, ignore_group_pairs, group_vec)

    def name(self) -> str:
        return "UniformWeeksChadlerAndersen"  # the reference's spelling

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_uniform_weeks_chandler_andersen(
            h, self.eps, self.sigma, len(self.former), i64ptr(self.former), len(self.latter),
            i64ptr(self.latter), *self._tail(self.system_size), C.byref(g)))
        return g.value


class UniformLennardJonesAttractiveForceFieldGenerator(_UniformPairGenerator):
    """The attractive Lennard-Jones form with one sigma and epsilon between
    `former` and `latter`; cutoff sigma * cutoff_ratio, switched from 0.9
    cutoff."""

    def __init__(self, system_size, eps, sigma, cutoff_ratio, former_group_vec, latter_group_vec,
                 ignore_list, use_periodic: bool, ignore_group_pairs=(), group_vec=()):
        self._uniform(system_size, eps, sigma, former_group_vec, latter_group_vec)
        self.cutoff_ratio = float(cutoff_ratio)
        self._common(ignore_list, use_periodic, ignore_group_pairs, group_vec)

    def name(self) -> str:
        return "UniformLennardJonesAttractive"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_uniform_lennard_jones_attractive(
            h, self.eps, self.sigma, self.cutoff_ratio, len(self.former), i64ptr(self.former),
            len(self.latter), i64ptr(self.latter), *self._tail(self.system_size), C.byref(g)))
        return g.value


class CappedGoContactForceFieldGenerator(_Generator):
    """The Go 10-12 form beyond capping_ratio * r0, its linear continuation
    (value and slope matched) below."""

    def __init__(self, indices_vec, ks, r0s, capping_ratio: float, use_periodic: bool):
        self.indices = _pairs_arg(indices_vec, 2)
        self.ks, self.r0s = as_f64(ks), as_f64(r0s)
        self.capping_ratio = float(capping_ratio)
        self.use_periodic = bool(use_periodic)
        if not (len(self.indices) == len(self.ks) == len(self.r0s)):
            raise OCMError(1, "[error] CappedGoContactForceFieldGenerator : parameter number of "
                              f"indices_vec ({len(self.indices)}), k ({len(self.ks)}) and "
                              f"r0 ({len(self.r0s)}) is not matched.The number of these parameters must be same.")

    def name(self) -> str:
        return "CappedGoContact"

    def add_to(self, h) -> int:
        g = C.c_int32()
        check(lib.ocm_add_capped_go_contact(h, len(self.indices), i64ptr(self.indices), dptr(self.ks),
                                            dptr(self.r0s), self.capping_ratio, int(self.use_periodic),
                                            C.byref(g)))
        return g.value


# ---------------------------------------------------------------------------
class System:
    """A generated system (owns the C handle)."""

    def __init__(self, handle, n: int):
        self._h = handle
        self.n = n

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.ocm_system_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def getNumParticles(self) -> int:
        return int(lib.ocm_system_num_particles(self._h))

    def num_groups(self) -> int:
        return int(lib.ocm_system_num_groups(self._h))

    def group_name(self, g: int) -> str:
        buf = C.create_string_buffer(256)
        check(lib.ocm_system_group_name(self._h, int(g), buf, 256))
        return buf.value.decode()

    def group_names(self) -> list[str]:
        return [self.group_name(g) for g in range(self.num_groups())]

    def describe(self) -> dict:
        need = C.c_int64()
        check(lib.ocm_system_describe(self._h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        check(lib.ocm_system_describe(self._h, buf, need.value, C.byref(need)))
        return json.loads(buf.value.decode())

    def footprint(self) -> int:
        return int(lib.ocm_batch_footprint(self._h))


class SystemGenerator:
    """Collects generators and assigns force groups (SystemGenerator.cpp:4-111)."""

    def __init__(self, mass_vec):
        self.masses = as_f64(mass_vec)
        self.generators: list[_Generator] = []
        self.pbc: tuple[float, float, float] | None = None

    def add_ff_generator(self, gen: _Generator) -> None:
        self.generators.append(gen)

    def set_pbc(self, x: float, y: float, z: float) -> None:
        self.pbc = (float(x), float(y), float(z))

    def generate(self) -> System:
        h = C.c_void_p()
        check(lib.ocm_system_create(len(self.masses), dptr(self.masses), C.byref(h)))
        sysobj = System(h, len(self.masses))
        if self.pbc is not None:
            check(lib.ocm_system_set_pbc(h, *self.pbc))
        for g in self.generators:
            g.add_to(h)
        return sysobj


class LangevinIntegrator:
    def __init__(self, temperature: float, friction: float, step_size: float, seed: int = 0):
        self.temperature, self.friction = float(temperature), float(friction)
        self.step_size, self.seed = float(step_size), int(seed)


class LangevinIntegratorGenerator:
    """LangevinIntegrator(T, gamma, dt) + setRandomNumberSeed (IntegratorGenerator.cpp:5-14)."""

    def __init__(self, temperature: float, friction_coeff: float, delta_t: float, seed: int):
        self._t, self._g, self._dt, self._seed = float(temperature), float(friction_coeff), float(delta_t), int(seed)

    def generate(self) -> LangevinIntegrator:
        return LangevinIntegrator(self._t, self._g, self._dt, self._seed)

    def temperature(self) -> float:
        return self._t

    def dump_info(self) -> str:
        seed = "not specified or 0. random seed will be chosen." if self._seed == 0 else f"{self._seed:7}"
        return (f"    temperature : {self._t:7.2f} K\n    delta_t     : {self._dt:7.3f} ps\n"
                f"    gamma       : {self._g:7.3f} ps^-1\n    seed        : {seed}")


def cutoff_ratio_for(absolute_nm: float, values: Sequence[float], lj: bool = False) -> float:
    """Ratio that makes a generator's cutoff equal ``absolute_nm``: EXV uses
    ratio * (max + 2nd max); LJ uses ratio * (max + 2nd max) / 2."""
    v = sorted((x for x in values if not math.isnan(x)), reverse=True)
    top = v[0] + (v[1] if len(v) > 1 else np.finfo(float).tiny)
    return absolute_nm / (0.5 * top if lj else top)
