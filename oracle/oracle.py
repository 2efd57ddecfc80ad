"""TEST INFRASTRUCTURE - ctypes front end of the FP64 CPU oracle
(oracle/ocm_oracle.cpp).  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, as the checker.  Parity unpinned: the
reference ships no golden vectors; the oracle is pinned by analytic
known-answer tests.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_I8 = C.POINTER(C.c_int8)


class OracleSystem(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("pos", _D), ("periodic", C.c_int), ("box", C.c_double * 3),
        ("n_bonds", C.c_int64), ("bond_idx", _I64), ("bond_v0", _D), ("bond_k", _D),
        ("bond_periodic", C.c_int),
        ("n_go", C.c_int64), ("go_idx", _I64), ("go_k", _D), ("go_r0", _D), ("go_periodic", C.c_int),
        ("n_fla", C.c_int64), ("fla_idx", _I64), ("fla_k", _D), ("fla_aa", _I32),
        ("n_fld", C.c_int64), ("fld_idx", _I64), ("fld_k", _D), ("fld_aa1", _I32), ("fld_aa2", _I32),
        ("exv_on", C.c_int), ("exv_eps", C.c_double), ("exv_ratio", C.c_double), ("exv_radius", _D),
        ("exv_ign_bond", C.c_int), ("exv_ign_contact", C.c_int),
        ("dh_on", C.c_int), ("dh_I", C.c_double), ("dh_T", C.c_double), ("dh_ratio", C.c_double),
        ("dh_q", _D), ("dh_ign_bond", C.c_int), ("dh_ign_contact", C.c_int),
        ("ljr_on", C.c_int), ("ljr_ratio", C.c_double), ("ljr_eps", _D), ("ljr_sigma", _D),
        ("ljr_ign_bond", C.c_int), ("ljr_ign_contact", C.c_int),
        ("lja_on", C.c_int), ("lja_ratio", C.c_double), ("lja_eps", _D), ("lja_sigma", _D),
        ("lja_ign_bond", C.c_int), ("lja_ign_contact", C.c_int),
        ("fp32_cutoff", C.c_int), ("pair_cells", C.c_int),
        ("n_gb", C.c_int64), ("gb_idx", _I64), ("gb_k", _D), ("gb_v0", _D), ("gb_sigma", _D),
        ("gb_periodic", C.c_int),
        ("n_gd", C.c_int64), ("gd_idx", _I64), ("gd_k", _D), ("gd_theta0", _D), ("gd_sigma", _D),
        ("gd_periodic", C.c_int),
        ("ljr_geometric", C.c_int), ("ljr_side", _I8), ("lja_side", _I8),
        ("n_cgo", C.c_int64), ("cgo_idx", _I64), ("cgo_k", _D), ("cgo_r0", _D), ("cgo_cap", _D),
        ("cgo_periodic", C.c_int), ("cgo_contact_edges", C.c_int),
        ("grp", _I32), ("n_igp", C.c_int64 * 4), ("igp", _I32 * 4), ("ign_molecule", C.c_int * 4),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.oracle_evaluate.argtypes = [C.POINTER(OracleSystem), _D, _D]
        L.oracle_evaluate.restype = C.c_int
        L.oracle_dh_params.argtypes = [C.c_double, C.c_double, C.c_double, _D]
        L.oracle_fla_min_energy.argtypes = [C.c_int]
        L.oracle_fla_min_energy.restype = C.c_double
        L.oracle_fld_min_energy.argtypes = [C.c_int]
        L.oracle_fld_min_energy.restype = C.c_double
        L.oracle_natural_spline.argtypes = [_D, C.c_double, _D]
        L.oracle_fld_classes.argtypes = [C.c_int, C.c_int, _I32, C.c_int]
        L.oracle_fld_classes.restype = C.c_int
        L.oracle_ignore_within.argtypes = [C.c_int64, C.c_int64, _I64, C.c_int64, _I64, C.c_int,
                                           C.c_int, _I64, C.c_int64, _I64]
        L.oracle_langevin_step.argtypes = [C.c_int64, _D, _D, _D, _D, C.c_double, C.c_double,
                                           C.c_double, C.c_uint32, C.c_uint32, C.c_uint64]
        L.oracle_simulate.argtypes = [C.POINTER(OracleSystem), _D, _D, _D, C.c_double, C.c_double,
                                      C.c_double, C.c_uint32, C.c_uint64, C.c_int64]
        L.oracle_gaussian3.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, _D]
        L.oracle_gaussian3.restype = None
        L.cpu_prepare.argtypes = [C.POINTER(OracleSystem), _D, _D, C.c_double, C.c_double, C.c_double,
                                  C.c_uint32, C.POINTER(C.c_void_p)]
        L.cpu_run_many.argtypes = [C.POINTER(C.c_void_p), C.c_int64, C.c_int64, C.c_int]
        L.cpu_evaluate.argtypes = [C.c_void_p, _D, _D]
        L.cpu_get_positions.argtypes = [C.c_void_p, _D]
        L.cpu_free.argtypes = [C.c_void_p]
        L.cpu_free.restype = None
        L.cpu_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _d(a):
    return None if a is None else np.ascontiguousarray(a, np.float64)


class _Keep:
    """Holds the numpy buffers an OracleSystem points into."""

    def __init__(self):
        self.items = []

    def d(self, a):
        if a is None:
            return None
        arr = np.ascontiguousarray(a, np.float64)
        self.items.append(arr)
        return arr.ctypes.data_as(_D)

    def i64(self, a):
        arr = np.ascontiguousarray(a, np.int64)
        self.items.append(arr)
        return arr.ctypes.data_as(_I64)

    def i8(self, a):
        if a is None:
            return None
        arr = np.ascontiguousarray(a, np.int8)
        self.items.append(arr)
        return arr.ctypes.data_as(_I8)

    def i32(self, a):
        arr = np.ascontiguousarray(a, np.int32)
        self.items.append(arr)
        return arr.ctypes.data_as(_I32)


def make_system(spec, fp32_cutoff: bool = True, pos=None, cells: int = -1):
    """Translate a synth.CGSpec into the oracle's flat description."""
    k = _Keep()
    s = OracleSystem()
    s.n = spec.n
    s.pos = k.d(spec.pos if pos is None else pos)
    s.periodic = int(spec.periodic)
    if spec.box is not None:
        for c in range(3):
            s.box[c] = spec.box[c]
    s.n_bonds = len(spec.bonds)
    s.bond_idx, s.bond_v0, s.bond_k = k.i64(spec.bonds), k.d(spec.bond_v0), k.d(spec.bond_k)
    s.bond_periodic = int(spec.periodic)
    s.n_go = len(spec.contacts)
    s.go_idx, s.go_k, s.go_r0 = k.i64(spec.contacts), k.d(spec.go_k), k.d(spec.go_r0)
    s.go_periodic = int(spec.periodic)
    s.n_fla = len(spec.fla_idx)
    s.fla_idx, s.fla_k, s.fla_aa = k.i64(spec.fla_idx), k.d(spec.fla_k), k.i32(spec.fla_aa)
    s.n_fld = len(spec.fld_idx)
    s.fld_idx, s.fld_k = k.i64(spec.fld_idx), k.d(spec.fld_k)
    s.fld_aa1, s.fld_aa2 = k.i32(spec.fld_aa1), k.i32(spec.fld_aa2)
    if spec.exv is not None:
        t = spec.exv
        s.exv_on, s.exv_eps, s.exv_ratio, s.exv_radius = 1, t.eps, t.ratio, k.d(t.p0)
        s.exv_ign_bond, s.exv_ign_contact = t.ign_bond, t.ign_contact
    if spec.dh is not None:
        t = spec.dh
        s.dh_on, s.dh_I, s.dh_T, s.dh_ratio, s.dh_q = 1, t.ionic_strength, t.temperature, t.ratio, k.d(t.p0)
        s.dh_ign_bond, s.dh_ign_contact = t.ign_bond, t.ign_contact
    if spec.ljr is not None:
        t = spec.ljr
        kind = getattr(t, "kind", "")
        # WCA forms (per-particle and uniform) cut off at 2^(1/6) sigma
        ratio = 2.0 ** (1.0 / 6.0) if kind in ("wca", "uniform") else t.ratio
        s.ljr_on, s.ljr_ratio, s.ljr_eps, s.ljr_sigma = 1, ratio, k.d(t.p0), k.d(t.p1)
        s.ljr_ign_bond, s.ljr_ign_contact = t.ign_bond, t.ign_contact
        s.ljr_geometric = int(kind == "wca")
        s.ljr_side = k.i8(getattr(t, "side", None))
    if spec.lja is not None:
        t = spec.lja
        s.lja_on, s.lja_ratio, s.lja_eps, s.lja_sigma = 1, t.ratio, k.d(t.p0), k.d(t.p1)
        s.lja_ign_bond, s.lja_ign_contact = t.ign_bond, t.ign_contact
        s.lja_side = k.i8(getattr(t, "side", None))
    s.fp32_cutoff = int(fp32_cutoff)
    s.pair_cells = int(cells)
    gb = getattr(spec, "gb_idx", np.zeros((0, 2), np.int64))
    s.n_gb = len(gb)
    if s.n_gb:
        s.gb_idx, s.gb_k, s.gb_v0, s.gb_sigma = k.i64(gb), k.d(spec.gb_k), k.d(spec.gb_v0), k.d(spec.gb_sigma)
    s.gb_periodic = int(spec.periodic)
    gd = getattr(spec, "gd_idx", np.zeros((0, 4), np.int64))
    s.n_gd = len(gd)
    if s.n_gd:
        s.gd_idx, s.gd_k = k.i64(gd), k.d(spec.gd_k)
        s.gd_theta0, s.gd_sigma = k.d(spec.gd_theta0), k.d(spec.gd_sigma)
    s.gd_periodic = int(spec.periodic)
    cgo = getattr(spec, "cgo_idx", np.zeros((0, 2), np.int64))
    s.n_cgo = len(cgo)
    if s.n_cgo:
        s.cgo_idx, s.cgo_k, s.cgo_r0 = k.i64(cgo), k.d(spec.cgo_k), k.d(spec.cgo_r0)
        s.cgo_cap = k.d(np.broadcast_to(np.asarray(spec.cgo_cap, float), (len(cgo),)))
    s.cgo_periodic = int(spec.periodic)
    s.cgo_contact_edges = int(getattr(spec, "cgo_topology", "none") == "contact")
    names = getattr(spec, "group_names", None)
    terms = (spec.exv, spec.dh, spec.ljr, spec.lja)
    for q, t in enumerate(terms):
        s.ign_molecule[q] = int(t is not None and getattr(t, "ign_molecule", False))
    if names is not None and any(t is not None and getattr(t, "ignore_groups", None) for t in terms):
        ids = {nm: q for q, nm in enumerate(sorted({g for g in names if g is not None}))}
        s.grp = k.i32([ids[g] if g is not None else -1 for g in names])
        for q, t in enumerate(terms):
            pairs = list(getattr(t, "ignore_groups", None) or []) if t is not None else []
            pairs = [(a, b) for a, b in pairs if a in ids and b in ids]  # a name nobody has ignores nothing
            s.n_igp[q] = len(pairs)
            if pairs:
                s.igp[q] = k.i32([ids[v] for p in pairs for v in p])
    return s, k


SLOTS = ("ExcludedVolume", "DebyeHuckel", "LennardJonesRepulsive", "LennardJonesAttractive",
         "HarmonicBond", "GoContact", "FlexibleLocalAngle", "FlexibleLocalDihedral", "GaussianBond",
         "GaussianDihedral", "CappedGoContact")


def slot_names(spec):
    """Force-group name of every energy slot for this spec (the Lennard-Jones
    slots carry the WCA and uniform variants under their own names)."""
    names = list(SLOTS)
    kind_r = getattr(spec.ljr, "kind", "") if spec.ljr is not None else ""
    kind_a = getattr(spec.lja, "kind", "") if spec.lja is not None else ""
    if kind_r == "wca":
        names[2] = "WeeksChandlerAndersen"
    elif kind_r == "uniform":
        names[2] = "UniformWeeksChadlerAndersen"
    if kind_a == "uniform":
        names[3] = "UniformLennardJonesAttractive"
    return tuple(names)


def evaluate(spec, fp32_cutoff: bool = True, pos=None, cells: int = -1):
    """FP64 forces (n, 3) and per-term energies {name: kJ/mol}.  Pairs are
    enumerated over all pairs (cells=0) or a cell grid (cells=1; -1 picks
    the grid above 4096 beads)."""
    s, keep = make_system(spec, fp32_cutoff, pos, cells)
    f = np.zeros((spec.n, 3))
    e = np.zeros(len(SLOTS))
    lib().oracle_evaluate(C.byref(s), f.ctypes.data_as(_D), e.ctypes.data_as(_D))
    del keep
    return f, dict(zip(slot_names(spec), e))


def dh_params(ionic_strength, temperature, ratio):
    out = np.zeros(5)
    lib().oracle_dh_params(ionic_strength, temperature, ratio, out.ctypes.data_as(_D))
    return dict(zip(("k_e", "debye_length", "cutoff", "cutoff_correction", "eps_r"), out))


def fla_min_energy(aa: int) -> float:
    return lib().oracle_fla_min_energy(int(aa))


def fld_min_energy(cls: int) -> float:
    return lib().oracle_fld_min_energy(int(cls))


def natural_spline(y, h):
    y = np.ascontiguousarray(y, np.float64)
    M = np.zeros(10)
    lib().oracle_natural_spline(y.ctypes.data_as(_D), h, M.ctypes.data_as(_D))
    return M


def fld_classes(aa1: int, aa2: int) -> list[int]:
    out = np.zeros(4, np.int32)
    c = lib().oracle_fld_classes(aa1, aa2, out.ctypes.data_as(_I32), 4)
    return [int(v) for v in out[:c]]


def ignore_within(n, bonds, contacts, ign_bond, ign_contact):
    b = np.ascontiguousarray(bonds, np.int64).reshape(-1, 2)
    c = np.ascontiguousarray(contacts, np.int64).reshape(-1, 2)
    cap = max(16, 64 * n)
    out = np.zeros((cap, 2), np.int64)
    nout = C.c_int64()
    lib().oracle_ignore_within(n, len(b), b.ctypes.data_as(_I64), len(c), c.ctypes.data_as(_I64),
                               ign_bond, ign_contact, out.ctypes.data_as(_I64), cap, C.byref(nout))
    return out[: nout.value].copy()


def langevin_step(x, v, f, masses, T, gamma, dt, seed, step, stream=0):
    x = np.ascontiguousarray(x, np.float64).copy()
    v = np.ascontiguousarray(v, np.float64).copy()
    f = np.ascontiguousarray(f, np.float64)
    m = np.ascontiguousarray(masses, np.float64)
    lib().oracle_langevin_step(len(m), x.ctypes.data_as(_D), v.ctypes.data_as(_D), f.ctypes.data_as(_D),
                               m.ctypes.data_as(_D), T, gamma, dt, seed, stream, step)
    return x, v


def simulate(spec, x, v, steps, seed, step0=0):
    """CPU baseline: `steps` oracle steps of one system (in place)."""
    s, keep = make_system(spec, fp32_cutoff=False, pos=x)
    m = np.ascontiguousarray(spec.masses, np.float64)
    lib().oracle_simulate(C.byref(s), x.ctypes.data_as(_D), v.ctypes.data_as(_D), m.ctypes.data_as(_D),
                          spec.temperature, spec.friction, spec.dt, seed, step0, steps)
    del keep


def gaussian3(seed, stream, bead, step, purpose=0):
    g = np.zeros(3)
    lib().oracle_gaussian3(seed, stream, bead, step, purpose, g.ctypes.data_as(_D))
    return g


class CpuEnsemble:
    """The timed CPU baseline (cpu_baseline.cpp): an FP32, Verlet-list,
    OpenMP restatement of the same force field and integrator, holding an
    ensemble of systems.  Set-up happens here (untimed); ``run`` advances
    every system by ``steps`` Langevin steps on ``threads`` host threads (0:
    all).  Not the reference (OpenMM is not installed) and not the checker:
    it exists to be timed."""

    def __init__(self, specs, seeds=None, velocities=None):
        L = lib()
        self.n = [int(sp.n) for sp in specs]
        self._h = (C.c_void_p * len(specs))()
        for k, sp in enumerate(specs):
            s, keep = make_system(sp, fp32_cutoff=False)
            m = np.ascontiguousarray(sp.masses, np.float64)
            v = None if velocities is None else np.ascontiguousarray(velocities[k], np.float64)
            seed = 1000 + k if seeds is None else int(seeds[k])
            h = C.c_void_p()
            code = L.cpu_prepare(C.byref(s), None if v is None else v.ctypes.data_as(_D), m.ctypes.data_as(_D),
                                 float(sp.temperature), float(sp.friction), float(sp.dt), seed, C.byref(h))
            del keep
            if code != 0:
                self.close()
                raise ValueError(f"system {k}: a feature the CPU restatement does not cover (code {code})")
            self._h[k] = h

    @staticmethod
    def max_threads() -> int:
        return int(lib().cpu_max_threads())

    def run(self, steps: int, threads: int = 0) -> None:
        lib().cpu_run_many(self._h, len(self.n), int(steps), int(threads))

    def evaluate(self, k: int):
        """FP32 forces (n, 3) and the EXV, DH, LJR, LJA, HB, GO, FLA, FLD energies."""
        f = np.zeros((self.n[k], 3))
        e = np.zeros(8)
        lib().cpu_evaluate(self._h[k], f.ctypes.data_as(_D), e.ctypes.data_as(_D))
        return f, e

    def positions(self, k: int) -> np.ndarray:
        x = np.zeros((self.n[k], 3))
        lib().cpu_get_positions(self._h[k], x.ctypes.data_as(_D))
        return x

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is None:
            return
        for k in range(len(h)):
            if h[k]:
                lib().cpu_free(h[k])
                h[k] = None
        self._h = None

    def __del__(self):
        self.close()
