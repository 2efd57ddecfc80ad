"""Seeded synthetic coarse-grained systems with the shapes of the benchmark
configurations, and their assembly through the reference-named generators.

No public dataset is involved: every system here is generated from a seed.
* Go-model protein: one chain of N beads from a self-avoiding random walk
  with 0.38 nm bonds; Go contacts on native pairs within 0.65 nm with
  |i-j| > 3 (eps ~ U[0.2, 1.0] kcal/mol); FLA/FLD from a random amino-acid
  sequence; EXV radius ~ U[0.2, 0.4] nm with a 2.0 nm cutoff; charges +-1 on
  25 % of beads with a 2.0 nm Debye-Hueckel cutoff; residue masses.
* HPS condensate slab: chains of 20 bead types (sigma ~ U[0.45, 0.75] nm,
  lambda ~ U[0, 1]) packed into the central slab of a periodic box; HPS
  Lennard-Jones with a 2.0 nm cutoff, Debye-Hueckel with 3.5 nm on 20 %
  charged beads, k = 10 kcal/mol/A^2 bonds.
Positions are rounded to FP32-representable values so the FP64 oracle and
the FP32 kernels see identical coordinates.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .forcefield import (AMINO_ACIDS, CappedGoContactForceFieldGenerator, DebyeHuckelForceFieldGenerator,
                         ExcludedVolumeForceFieldGenerator, FlexibleLocalAngleForceFieldGenerator,
                         FlexibleLocalDihedralForceFieldGenerator, GaussianBondForceFieldGenerator,
                         GaussianDihedralForceFieldGenerator, GoContactForceFieldGenerator,
                         HarmonicBondForceFieldGenerator, LennardJonesAttractiveForceFieldGenerator,
                         LennardJonesRepulsiveForceFieldGenerator, System, SystemGenerator,
                         Topology, UniformLennardJonesAttractiveForceFieldGenerator,
                         UniformWeeksChandlerAndersenForceFieldGenerator,
                         WeeksChandlerAndersenForceFieldGenerator, fla_spline_table, fld_fourier_table,
                         fld_table_keys)

KJ_PER_KCAL = 4.184
ANGSTROM_PER_NM = 10.0
BOLTZ = 0.00831446261815324  # kJ/mol/K

# Average residue masses (amu) of the 20 amino acids, AMINO_ACIDS order.
RESIDUE_MASS = np.array([71.08, 156.19, 114.10, 115.09, 103.14, 128.13, 129.12, 57.05, 137.14,
                         113.16, 113.16, 128.17, 131.19, 147.18, 97.12, 87.08, 101.10, 186.21,
                         163.18, 99.13])


@dataclass
class PairTerm:
    ratio: float
    p0: np.ndarray                     # radius / charge / epsilon (NaN = absent)
    p1: np.ndarray | None = None       # sigma for LJ terms
    eps: float = 0.0                   # EXV epsilon (kJ/mol)
    ionic_strength: float = 0.15
    temperature: float = 300.0
    ign_bond: int = -1                 # exclusions within this many bonds (-1: none)
    ign_contact: int = -1              # exclusions within this many contacts
    ign_molecule: bool = False         # exclude every pair inside one molecule (bond-connected)
    # Lennard-Jones slot variants: "" (the HPS generators), "wca"
    # (WeeksChandlerAndersen, repulsive slot), "uniform" (the uniform
    # generators: p0 / p1 hold one epsilon / sigma, `side` marks the
    # former (bit 1) and latter (bit 2) particle lists)
    kind: str = ""
    side: np.ndarray | None = None
    # group-based ignores: (name, name) pairs of the particles' group names
    # (CGSpec.group_names) whose pairs do not interact
    ignore_groups: list | None = None


@dataclass
class CGSpec:
    n: int
    pos: np.ndarray
    masses: np.ndarray
    periodic: bool = False
    box: tuple | None = None
    bonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    bond_v0: np.ndarray = field(default_factory=lambda: np.zeros(0))
    bond_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    contacts: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    go_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    go_r0: np.ndarray = field(default_factory=lambda: np.zeros(0))
    fla_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int64))
    fla_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    fla_aa: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    fld_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int64))
    fld_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    fld_aa1: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    fld_aa2: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    # AICG2+ Gaussian bonds (k kJ/mol, v0 and sigma nm) and dihedrals
    # (k kJ/mol, theta0 and sigma rad)
    gb_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    gb_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    gb_v0: np.ndarray = field(default_factory=lambda: np.zeros(0))
    gb_sigma: np.ndarray = field(default_factory=lambda: np.zeros(0))
    gd_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int64))
    gd_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    gd_theta0: np.ndarray = field(default_factory=lambda: np.zeros(0))
    gd_sigma: np.ndarray = field(default_factory=lambda: np.zeros(0))
    # capped Go contacts: capping ratio (one for all, or one per contact),
    # and whether they are "contact" edges of the topology (exclusions)
    cgo_idx: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    cgo_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    cgo_r0: np.ndarray = field(default_factory=lambda: np.zeros(0))
    cgo_cap: float | np.ndarray = 0.8
    cgo_topology: str = "none"
    group_names: list | None = None  # per-particle group name (None: no group)
    exv: PairTerm | None = None
    dh: PairTerm | None = None
    ljr: PairTerm | None = None
    lja: PairTerm | None = None
    temperature: float = 300.0
    friction: float = 0.1
    dt: float = 0.01


def debye_length(temperature: float, ionic_strength: float) -> float:
    """Debye length (nm) by the reference's formula (DebyeHuckelForceFieldGenerator.cpp:22-43)."""
    eps_r = DebyeHuckelForceFieldGenerator.dielectric_water(temperature, ionic_strength)
    na, kb, e = 6.02214076e23, 1.380649e-23, 1.6021766208e-19
    eps0 = 8.854187817e-12 * 1.0e3 * 1.0e-9 / na / e / e
    return math.sqrt((eps0 * eps_r * kb * 1.0e-3 * temperature) / (2.0 * ionic_strength * 1.0e-24))


def _f32(a: np.ndarray) -> np.ndarray:
    return np.asarray(a, np.float32).astype(np.float64)


def _cross(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """a x b of two 3-vectors (the products np.cross forms, without its
    per-call overhead)."""
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])


def _orthonormal(b: np.ndarray):
    t = np.array([1.0, 0.0, 0.0]) if abs(b[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = _cross(b, t)
    u /= np.linalg.norm(u)
    return u, _cross(b, u)


def saw_chain(n: int, rng: np.random.Generator, bond: float = 0.38, min_dist: float = 0.45,
              theta=(1.75, 2.6)) -> np.ndarray:
    """Self-avoiding random walk: bond angles in `theta` (rad), beads at least
    `min_dist` from every earlier non-adjacent bead."""
    for _attempt in range(100):
        x = np.zeros((n, 3))
        if n > 1:
            d = rng.normal(size=3)
            x[1] = bond * d / np.linalg.norm(d)
        ok = True
        for i in range(2, n):
            b = x[i - 1] - x[i - 2]
            b /= np.linalg.norm(b)
            u, w = _orthonormal(b)
            placed = False
            for _try in range(200):
                th = rng.uniform(*theta)
                ph = rng.uniform(-math.pi, math.pi)
                dvec = -math.cos(th) * b + math.sin(th) * (math.cos(ph) * u + math.sin(ph) * w)
                cand = x[i - 1] + bond * dvec
                if i >= 3:
                    dd = np.min(np.sum((x[: i - 1] - cand) ** 2, axis=1))
                    if dd < min_dist * min_dist:
                        continue
                x[i] = cand
                placed = True
                break
            if not placed:
                ok = False
                break
        if ok:
            return x
    raise RuntimeError("could not grow a self-avoiding chain")


def go_protein(n: int, seed: int, temperature: float = 300.0, cutoff: float = 2.0,
               charge_fraction: float = 0.25, ionic_strength: float = 0.15,
               exv_eps_kcal: float = 0.6, contact_cutoff: float = 0.65) -> CGSpec:
    rng = np.random.default_rng(seed)
    seq = rng.integers(0, 20, n).astype(np.int32)
    pos = _f32(saw_chain(n, rng))
    s = CGSpec(n=n, pos=pos, masses=RESIDUE_MASS[seq].copy(), temperature=temperature)
    s.bonds = np.stack([np.arange(n - 1), np.arange(1, n)], 1).astype(np.int64)
    s.bond_v0 = np.linalg.norm(pos[1:] - pos[:-1], axis=1)
    s.bond_k = np.full(n - 1, 110.0 * KJ_PER_KCAL * ANGSTROM_PER_NM ** 2 * 2.0)
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=2)
    ii, jj = np.nonzero(np.triu(d < contact_cutoff, k=4))
    s.contacts = np.stack([ii, jj], 1).astype(np.int64)
    s.go_k = rng.uniform(0.2, 1.0, len(ii)) * KJ_PER_KCAL
    s.go_r0 = d[ii, jj]
    if n >= 3:
        c = np.arange(1, n - 1)
        s.fla_idx = np.stack([c - 1, c, c + 1], 1).astype(np.int64)
        s.fla_k = np.full(n - 2, 1.0 * KJ_PER_KCAL)
        s.fla_aa = seq[c]
    if n >= 4:
        c = np.arange(1, n - 2)
        s.fld_idx = np.stack([c - 1, c, c + 1, c + 2], 1).astype(np.int64)
        s.fld_k = np.full(n - 3, 1.0 * KJ_PER_KCAL)
        s.fld_aa1 = seq[c]
        s.fld_aa2 = seq[c + 1]
    radius = rng.uniform(0.2, 0.4, n)
    top = np.sort(radius)[::-1]
    s.exv = PairTerm(ratio=cutoff / (top[0] + top[1]), p0=radius, eps=exv_eps_kcal * KJ_PER_KCAL,
                     ign_bond=3, ign_contact=1)
    q = np.full(n, np.nan)
    nq = max(2, int(round(charge_fraction * n)))
    pick = rng.choice(n, nq, replace=False)
    q[pick] = rng.choice([-1.0, 1.0], nq)
    s.dh = PairTerm(ratio=cutoff / debye_length(temperature, ionic_strength), p0=q,
                    ionic_strength=ionic_strength, temperature=temperature, ign_bond=3)
    return s


def dihedral_angles(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """IUPAC dihedral angles (OpenMM's torsion convention) of quadruplets."""
    b1 = pos[idx[:, 1]] - pos[idx[:, 0]]
    b2 = pos[idx[:, 2]] - pos[idx[:, 1]]
    b3 = pos[idx[:, 3]] - pos[idx[:, 2]]
    n1, n2 = np.cross(b1, b2), np.cross(b2, b3)
    y = np.linalg.norm(b2, axis=1) * np.sum(b1 * n2, axis=1)
    return np.arctan2(y, np.sum(n1 * n2, axis=1))


def add_aicg_gaussians(spec: CGSpec, seed: int, gb_sigma: float = 0.015,
                       gd_sigma: float = 0.15) -> CGSpec:
    """Attach AICG2+-shaped Gaussian terms to a chain (as in the AICG2+
    sample inputs): bonds between beads i and i+2 centred on their current
    distance and dihedrals over i..i+3 centred on their current angle, with
    negative k (attractive wells) drawn from a seeded generator."""
    rng = np.random.default_rng(seed)
    n = spec.n
    if n >= 3:
        i = np.arange(n - 2)
        spec.gb_idx = np.stack([i, i + 2], 1).astype(np.int64)
        spec.gb_v0 = np.linalg.norm(spec.pos[i + 2] - spec.pos[i], axis=1)
        spec.gb_k = -rng.uniform(0.5, 1.5, n - 2) * KJ_PER_KCAL
        spec.gb_sigma = np.full(n - 2, gb_sigma)
    if n >= 4:
        i = np.arange(n - 3)
        spec.gd_idx = np.stack([i, i + 1, i + 2, i + 3], 1).astype(np.int64)
        spec.gd_theta0 = dihedral_angles(spec.pos, spec.gd_idx)
        spec.gd_k = -rng.uniform(0.2, 0.6, n - 3) * KJ_PER_KCAL
        spec.gd_sigma = np.full(n - 3, gd_sigma)
    return spec


def _pack_chains(n_chains: int, chain_len: int, L: np.ndarray, zlo: float, zhi: float, min_dist: float,
                 rng: np.random.Generator, bond: float = 0.38, theta=(1.75, 2.6)) -> np.ndarray:
    """Random-walk chains packed into the slab zlo <= z <= zhi of a periodic
    box, every bead at least ``min_dist`` from every other bead except its
    bonded predecessor.  All chains grow at once, one bead per chain per
    round: a chain proposes one candidate (eight after a failure), drawn
    with numpy (bond angle in ``theta`` after the second bead, a free
    direction after 400 failed tries); candidates are checked against the
    placed beads through a dense cell grid and against each other with a
    periodic k-d tree.  A chain stuck for 800 tries steps back eight beads;
    after 200 step-backs it starts over."""
    from scipy.spatial import cKDTree
    n = n_chains * chain_len
    nc = np.maximum(1, np.floor(L / min_dist).astype(np.int64))
    cw = L / nc
    cap = 4  # a cell is min_dist wide: at most three beads fit (one bonded pair closer)
    grid = np.full((int(np.prod(nc)), cap), -1, np.int64)
    gcnt = np.zeros(int(np.prod(nc)), np.int64)
    pos = np.full((n, 3), np.nan)
    wpos = np.full((n + 1, 3), np.nan, np.float32)  # wrapped into the box; row n: an empty slot
    length = np.zeros(n_chains, np.int64)
    prev_dir = np.zeros((n_chains, 3))
    tries = np.zeros(n_chains, np.int64)
    backs = np.zeros(n_chains, np.int64)
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    md2 = min_dist * min_dist

    def wrap(p):
        w = p - L * np.floor(p / L)
        return np.where(w >= L, w - L, w)

    def cells(p):
        return np.minimum((wrap(p) / cw).astype(np.int64), nc - 1)

    def lin(c):
        return (c[..., 0] * nc[1] + c[..., 1]) * nc[2] + c[..., 2]

    def insert(lc, gidx):
        order = np.argsort(lc, kind="stable")
        lcs, gs = lc[order], gidx[order]
        uniq, first, counts = np.unique(lcs, return_index=True, return_counts=True)
        rank = np.arange(len(lcs)) - np.repeat(first, counts)
        slot = gcnt[lcs] + rank
        if np.any(slot >= cap):
            raise RuntimeError("slab packing: a grid cell overflowed")
        grid[lcs, slot] = gs
        gcnt[uniq] += counts

    def drop_beads(c, keep):
        """Remove beads keep.. of chain c from the grid."""
        for g in range(c * chain_len + keep, c * chain_len + int(length[c])):
            cell = int(lin(cells(pos[g])))
            row = grid[cell, : gcnt[cell]]
            rest = row[row != g]
            grid[cell, :] = -1
            grid[cell, : len(rest)] = rest
            gcnt[cell] = len(rest)
            pos[g] = np.nan
            wpos[g] = np.nan
        length[c] = keep
        if keep >= 2:
            b = pos[c * chain_len + keep - 1] - pos[c * chain_len + keep - 2]
            b -= L * np.round(b / L)
            prev_dir[c] = b / np.linalg.norm(b)

    while True:
        act = np.nonzero(length < chain_len)[0]
        if act.size == 0:
            break
        ncand = np.where(tries[act] == 0, 1, 8)
        row = np.repeat(np.arange(act.size), ncand)      # candidate -> active chain
        ch = act[row]
        k = length[ch]
        m = row.size
        cand = np.empty((m, 3))
        dirs = np.zeros((m, 3))
        first = k == 0
        if first.any():
            f = int(first.sum())
            cand[first] = np.stack([rng.uniform(0, L[0], f), rng.uniform(0, L[1], f), rng.uniform(zlo, zhi, f)], 1)
        rest = np.nonzero(~first)[0]
        if rest.size:
            d = rng.normal(size=(rest.size, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            con = (k[rest] >= 2) & (tries[ch[rest]] < 400)
            if con.any():
                b = prev_dir[ch[rest[con]]]
                t = np.where(np.abs(b[:, :1]) < 0.9, np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0]))
                u = np.cross(b, t)
                u /= np.linalg.norm(u, axis=1, keepdims=True)
                w = np.cross(b, u)
                th = rng.uniform(theta[0], theta[1], len(b))[:, None]
                ph = rng.uniform(-math.pi, math.pi, len(b))[:, None]
                d[con] = -np.cos(th) * b + np.sin(th) * (np.cos(ph) * u + np.sin(ph) * w)
            dirs[rest] = d
            cand[rest] = pos[ch[rest] * chain_len + k[rest] - 1] + bond * d
        ok = (cand[:, 2] >= zlo) & (cand[:, 2] <= zhi)
        wc = wrap(cand)
        cc = np.minimum((wc / cw).astype(np.int64), nc - 1)
        raw = cc[:, None, :] + offs[None, :, :]                                # (m, 27, 3)
        shift = (np.floor_divide(raw, nc) * L).astype(np.float32)              # image of each cell
        idx = grid[lin(raw % nc)]                                              # (m, 27, cap)
        own_prev = np.where(k > 0, ch * chain_len + k - 1, -2)
        idx = np.where(idx == own_prev[:, None, None], -1, idx)
        dd = wpos[np.where(idx >= 0, idx, n)] + (shift - wc[:, None, :].astype(np.float32))[:, :, None, :]
        d2 = np.einsum("mcsk,mcsk->mcs", dd, dd)
        ok &= ~np.any(d2 < np.float32(md2), axis=(1, 2))  # empty slots hold NaN: never close
        # each chain keeps its first valid candidate
        good = np.nonzero(ok)[0]
        _, firsts = np.unique(row[good], return_index=True)
        pick = good[firsts]
        if pick.size > 1:
            w = cand[pick] - L * np.floor(cand[pick] / L)
            w = np.where(w >= L, w - L, w)
            pairs = cKDTree(w, boxsize=L).query_pairs(min_dist, output_type="ndarray")
            if len(pairs):
                pick = np.delete(pick, np.unique(pairs.max(axis=1)))
        placed = np.zeros(act.size, bool)
        if pick.size:
            ca = ch[pick]
            gidx = ca * chain_len + k[pick]
            pos[gidx] = cand[pick]
            wpos[gidx] = wc[pick]
            prev_dir[ca] = dirs[pick]
            length[ca] += 1
            tries[ca] = 0
            insert(lin(cc[pick]), gidx)
            placed[row[pick]] = True
        fail = act[~placed]
        tries[fail] += ncand[~placed]
        for c in fail[tries[fail] > 800]:
            c = int(c)
            backs[c] += 1
            if backs[c] > 200:
                drop_beads(c, 0)
                backs[c] = 0
            else:
                drop_beads(c, max(0, int(length[c]) - 8))
            tries[c] = 0
    return pos


def hps_slab(n_chains: int, chain_len: int, box, slab_width: float, seed: int,
             hps_cutoff: float = 2.0, dh_cutoff: float = 3.5, charge_fraction: float = 0.2,
             ionic_strength: float = 0.15, temperature: float = 300.0,
             min_dist: float = 0.5) -> CGSpec:
    rng = np.random.default_rng(seed)
    box = tuple(float(b) for b in box)
    sig_t = rng.uniform(0.45, 0.75, 20)
    lam_t = rng.uniform(0.0, 1.0, 20)
    n = n_chains * chain_len
    types = rng.integers(0, 20, n).astype(np.int32)
    L = np.array(box)
    zlo, zhi = 0.5 * box[2] - 0.5 * slab_width, 0.5 * box[2] + 0.5 * slab_width
    pos = _pack_chains(n_chains, chain_len, L, zlo, zhi, min_dist, rng)
    pos = pos - L * np.floor(pos / L)
    pos = _f32(pos)
    pos = np.where(pos >= L, pos - L, pos)  # FP32 rounding may land exactly on L
    s = CGSpec(n=n, pos=pos, masses=RESIDUE_MASS[types].copy(), periodic=True, box=box,
               temperature=temperature)
    starts = np.arange(n_chains) * chain_len
    b0 = (starts[:, None] + np.arange(chain_len - 1)[None, :]).ravel()
    s.bonds = np.stack([b0, b0 + 1], 1).astype(np.int64)
    dv = pos[s.bonds[:, 1]] - pos[s.bonds[:, 0]]
    dv -= L * np.round(dv / L)
    s.bond_v0 = np.linalg.norm(dv, axis=1)
    s.bond_k = np.full(len(b0), 10.0 * KJ_PER_KCAL * ANGSTROM_PER_NM ** 2 * 2.0)
    sig = sig_t[types]
    lj_ratio = hps_cutoff / (0.5 * (np.sort(sig)[-1] + np.sort(sig)[-2]))
    s.ljr = PairTerm(ratio=lj_ratio, p0=np.full(n, 0.2 * KJ_PER_KCAL), p1=sig, ign_bond=1)
    s.lja = PairTerm(ratio=lj_ratio, p0=0.2 * lam_t[types] * KJ_PER_KCAL, p1=sig, ign_bond=1)
    q = np.full(n, np.nan)
    nq = max(2, int(round(charge_fraction * n)))
    pick = rng.choice(n, nq, replace=False)
    q[pick] = rng.choice([-1.0, 1.0], nq)
    s.dh = PairTerm(ratio=dh_cutoff / debye_length(temperature, ionic_strength), p0=q,
                    ionic_strength=ionic_strength, temperature=temperature, ign_bond=3)
    return s


def ensemble_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """Bead counts log-uniform in [lo, hi] (seeded)."""
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi + 1), count))).astype(int).clip(lo, hi)


def ensemble_temperatures(count: int, seed: int, lo: float = 280.0, hi: float = 360.0) -> np.ndarray:
    return np.random.default_rng(seed + 7919).uniform(lo, hi, count)


# ---------------------------------------------------------------------------
def fld_selects(key: str, a1: str, a2: str) -> bool:
    """Whether the reader assigns dihedral class `key` to a "a1-a2" coef
    (ReadTOMLForceFieldGenerator.cpp:637-744)."""
    first, second = key.split("-")
    if second == "GLY":
        return a2 == "GLY"
    if second == "PRO":
        return (a1 == "GLY" and a2 == "PRO") if first == "GLY" else a2 == "PRO"
    return a2 not in ("GLY", "PRO") and a1 == first


def _ignore(topo: Topology, bond: int, contact: int, molecule: bool = False) -> np.ndarray:
    parts = []
    if molecule:  # ignore.molecule = "Intra" / "Self": molecules from the bond edges
        topo.make_molecule("bond")
        parts.append(topo.ignore_list_within_molecule())
    if bond >= 0:
        parts.append(topo.ignore_list_within_edge(bond, "bond"))
    if contact >= 0:
        parts.append(topo.ignore_list_within_edge(contact, "contact"))
    if not parts:
        return np.zeros((0, 2), np.int64)
    allp = np.concatenate(parts)
    return np.unique(allp, axis=0) if len(allp) else allp


def build_generator(spec: CGSpec) -> SystemGenerator:
    """Assemble the spec through the reference-named generators, local
    forces first (harmonic, Go, Gaussian bond, FLA, Gaussian dihedral, FLD:
    the order of the AICG2+ sample inputs) and then the pair forces."""
    per = spec.periodic
    topo = Topology(spec.n)
    if len(spec.bonds):
        topo.add_edges(spec.bonds, "bond")
    if len(spec.contacts):
        topo.add_edges(spec.contacts, "contact")
    if len(spec.cgo_idx) and spec.cgo_topology == "contact":
        topo.add_edges(spec.cgo_idx, "contact")
    sg = SystemGenerator(spec.masses)
    if per:
        sg.set_pbc(*spec.box)
    if len(spec.bonds):
        sg.add_ff_generator(HarmonicBondForceFieldGenerator(spec.bonds, spec.bond_v0, spec.bond_k, per))
    if len(spec.contacts):
        sg.add_ff_generator(GoContactForceFieldGenerator(spec.contacts, spec.go_k, spec.go_r0, per))
    if len(spec.cgo_idx):
        caps = np.broadcast_to(np.asarray(spec.cgo_cap, float), (len(spec.cgo_idx),))
        for cap in np.unique(caps):  # one generator per capping ratio
            sel = caps == cap
            sg.add_ff_generator(CappedGoContactForceFieldGenerator(spec.cgo_idx[sel], spec.cgo_k[sel],
                                                                   spec.cgo_r0[sel], float(cap), per))
    if len(spec.gb_idx):
        sg.add_ff_generator(GaussianBondForceFieldGenerator(spec.gb_idx, spec.gb_k, spec.gb_v0,
                                                            spec.gb_sigma, per))
    if len(spec.fla_idx):
        for a, aa in enumerate(AMINO_ACIDS):
            sel = spec.fla_aa == a
            sg.add_ff_generator(FlexibleLocalAngleForceFieldGenerator(
                spec.fla_idx[sel], spec.fla_k[sel], fla_spline_table(aa), aa, per))
    if len(spec.gd_idx):
        sg.add_ff_generator(GaussianDihedralForceFieldGenerator(spec.gd_idx, spec.gd_k, spec.gd_theta0,
                                                                spec.gd_sigma, per))
    if len(spec.fld_idx):
        a1 = [AMINO_ACIDS[v] for v in spec.fld_aa1]
        a2 = [AMINO_ACIDS[v] for v in spec.fld_aa2]
        for key in fld_table_keys():
            sel = np.array([fld_selects(key, x, y) for x, y in zip(a1, a2)], bool)
            sg.add_ff_generator(FlexibleLocalDihedralForceFieldGenerator(
                spec.fld_idx[sel], spec.fld_k[sel], fld_fourier_table(key), key, per))
    def grp(t):  # group-based ignores of a pair term
        return dict(ignore_group_pairs=list(t.ignore_groups or ()),
                    group_vec=list(spec.group_names) if t.ignore_groups else ())

    if spec.exv is not None:
        t = spec.exv
        sg.add_ff_generator(ExcludedVolumeForceFieldGenerator(
            t.eps, t.ratio, t.p0, _ignore(topo, t.ign_bond, t.ign_contact, t.ign_molecule), per, **grp(t)))
    if spec.ljr is not None:
        t = spec.ljr
        ign = _ignore(topo, t.ign_bond, t.ign_contact, t.ign_molecule)
        if t.kind == "wca":
            sg.add_ff_generator(WeeksChandlerAndersenForceFieldGenerator(t.p1, t.p0, ign, per, **grp(t)))
        elif t.kind == "uniform":
            sg.add_ff_generator(UniformWeeksChandlerAndersenForceFieldGenerator(
                spec.n, t.p0[0], t.p1[0], np.nonzero(t.side & 1)[0], np.nonzero(t.side & 2)[0], ign, per,
                **grp(t)))
        else:
            sg.add_ff_generator(LennardJonesRepulsiveForceFieldGenerator(t.ratio, t.p0, t.p1, ign, per, **grp(t)))
    if spec.lja is not None:
        t = spec.lja
        ign = _ignore(topo, t.ign_bond, t.ign_contact, t.ign_molecule)
        if t.kind == "uniform":
            sg.add_ff_generator(UniformLennardJonesAttractiveForceFieldGenerator(
                spec.n, t.p0[0], t.p1[0], t.ratio, np.nonzero(t.side & 1)[0], np.nonzero(t.side & 2)[0],
                ign, per, **grp(t)))
        else:
            sg.add_ff_generator(LennardJonesAttractiveForceFieldGenerator(t.ratio, t.p0, t.p1, ign, per, **grp(t)))
    if spec.dh is not None:
        t = spec.dh
        sg.add_ff_generator(DebyeHuckelForceFieldGenerator(
            t.ionic_strength, t.temperature, t.ratio, t.p0, _ignore(topo, t.ign_bond, t.ign_contact, t.ign_molecule), per,
            **grp(t)))
    return sg


def build_system(spec: CGSpec) -> System:
    return build_generator(spec).generate()


# ---------------------------------------------------------------------------
_PAIR_KEYS = ("exv", "dh", "ljr", "lja")
_ARRAY_KEYS = ("pos", "masses", "bonds", "bond_v0", "bond_k", "contacts", "go_k", "go_r0", "fla_idx",
               "fla_k", "fla_aa", "fld_idx", "fld_k", "fld_aa1", "fld_aa2", "gb_idx", "gb_k", "gb_v0",
               "gb_sigma", "gd_idx", "gd_k", "gd_theta0", "gd_sigma", "cgo_idx", "cgo_k", "cgo_r0")


def spec_to_arrays(spec: CGSpec) -> dict:
    """Flat dict of numpy arrays (for ``np.savez``) describing a spec."""
    out = {k: np.asarray(getattr(spec, k)) for k in _ARRAY_KEYS}
    out["scalars"] = np.array([spec.n, int(spec.periodic), spec.temperature, spec.friction, spec.dt])
    out["box"] = np.asarray(spec.box if spec.box is not None else (0.0, 0.0, 0.0), float)
    out["cgo_cap"] = np.atleast_1d(np.asarray(spec.cgo_cap, float))
    for key in _PAIR_KEYS:
        t = getattr(spec, key)
        if t is None:
            continue
        out[f"{key}_p0"] = np.asarray(t.p0, float)
        if t.p1 is not None:
            out[f"{key}_p1"] = np.asarray(t.p1, float)
        out[f"{key}_scalars"] = np.array([t.ratio, t.eps, t.ionic_strength, t.temperature,
                                          t.ign_bond, t.ign_contact], float)
    return out


def spec_from_arrays(d) -> CGSpec:
    """Inverse of ``spec_to_arrays`` (accepts an ``np.load`` result)."""
    sc = d["scalars"]
    spec = CGSpec(n=int(sc[0]), pos=np.array(d["pos"], float), masses=np.array(d["masses"], float),
                  periodic=bool(sc[1]), temperature=float(sc[2]), friction=float(sc[3]), dt=float(sc[4]))
    if spec.periodic:
        spec.box = tuple(float(v) for v in d["box"])
    for k in _ARRAY_KEYS[2:]:
        if k in d:
            setattr(spec, k, np.array(d[k]))
    if "cgo_cap" in d:
        cap = np.asarray(d["cgo_cap"], float)
        spec.cgo_cap = float(cap[0]) if cap.size == 1 else cap
    for key in _PAIR_KEYS:
        if f"{key}_scalars" not in d:
            continue
        s = d[f"{key}_scalars"]
        setattr(spec, key, PairTerm(ratio=float(s[0]), p0=np.array(d[f"{key}_p0"], float),
                                    p1=np.array(d[f"{key}_p1"], float) if f"{key}_p1" in d else None,
                                    eps=float(s[1]), ionic_strength=float(s[2]), temperature=float(s[3]),
                                    ign_bond=int(s[4]), ign_contact=int(s[5])))
    return spec


def subset_spec(spec: CGSpec, n_keep: int) -> CGSpec:
    """The first ``n_keep`` beads of a spec with every term that lies
    entirely inside them (whole chains when ``n_keep`` ends a chain)."""
    import copy
    s = copy.deepcopy(spec)
    s.n = n_keep
    s.pos, s.masses = spec.pos[:n_keep].copy(), spec.masses[:n_keep].copy()

    def keep(idx):
        return np.all(idx < n_keep, axis=1) if len(idx) else np.zeros(0, bool)

    m = keep(spec.bonds)
    s.bonds, s.bond_v0, s.bond_k = spec.bonds[m], spec.bond_v0[m], spec.bond_k[m]
    m = keep(spec.contacts)
    s.contacts, s.go_k, s.go_r0 = spec.contacts[m], spec.go_k[m], spec.go_r0[m]
    m = keep(spec.fla_idx)
    s.fla_idx, s.fla_k, s.fla_aa = spec.fla_idx[m], spec.fla_k[m], spec.fla_aa[m]
    m = keep(spec.fld_idx)
    s.fld_idx, s.fld_k, s.fld_aa1, s.fld_aa2 = spec.fld_idx[m], spec.fld_k[m], spec.fld_aa1[m], spec.fld_aa2[m]
    m = keep(spec.gb_idx)
    s.gb_idx, s.gb_k, s.gb_v0, s.gb_sigma = spec.gb_idx[m], spec.gb_k[m], spec.gb_v0[m], spec.gb_sigma[m]
    m = keep(spec.gd_idx)
    s.gd_idx, s.gd_k, s.gd_theta0, s.gd_sigma = (spec.gd_idx[m], spec.gd_k[m], spec.gd_theta0[m],
                                                 spec.gd_sigma[m])
    m = keep(spec.cgo_idx)
    s.cgo_idx, s.cgo_k, s.cgo_r0 = spec.cgo_idx[m], spec.cgo_k[m], spec.cgo_r0[m]
    if np.ndim(spec.cgo_cap):
        s.cgo_cap = np.asarray(spec.cgo_cap)[m]
    for key in _PAIR_KEYS:
        t = getattr(s, key)
        if t is not None:
            t.p0 = t.p0[:n_keep].copy()
            if t.p1 is not None:
                t.p1 = t.p1[:n_keep].copy()
            if t.side is not None:
                t.side = t.side[:n_keep].copy()
    return s
