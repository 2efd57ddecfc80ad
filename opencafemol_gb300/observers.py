"""Trajectory and energy output in the reference's file formats, written by a
background thread.

The reference's ``Simulator::run`` (src/Simulator.cpp:50-76) calls every
observer at step ``frame * save_step`` before advancing ``save_step`` steps.
``Simulator`` below runs the same loop on a ``Context``.  Each observer reads
what it needs from the device at that step (one fused evaluation gives every
force group's energy, instead of one ``getState`` per group as in
src/Observer.cpp:332-347) and hands the numbers to a writer thread, so
formatting and disk writes overlap with the next steps.

File layouts follow src/Observer.cpp:
* ``<prefix>.ene``: "# unit of energy : kcal/mol", a column header with the
  force-group names in name order (the reference's std::map) and
  "kinetic_energy", then per frame the step (left-aligned, width 10), each
  group's energy (width 24, fixed, 6 decimals) and the kinetic energy
  (width 14), in kcal/mol;
* ``<prefix>_position.dcd`` / ``<prefix>_velocity.dcd``: CHARMM-style DCD
  (84-byte "CORD" block with frame count, save interval, total steps,
  delta_t, unit-cell flag and version 24; an 80-character title block; the
  particle count), then per frame an optional unit-cell record
  (A, gamma, B, beta, alpha, C as doubles, Angstrom and degrees) and the x,
  y and z records as float32, positions in Angstrom and velocities in
  Angstrom per cafetime;
* ``<prefix>.pdb``: MODEL/ATOM/ENDMDL frames in Angstrom.
"""
from __future__ import annotations

import math
import queue
import struct
import threading
from pathlib import Path

import numpy as np

KCAL_PER_KJ = 1.0 / 4.184
ANGSTROM_PER_NM = 10.0
CAFETIME_PS = math.sqrt(1.0 / 4.184) * 0.1
DCD_TITLE = b"written by opencafemol_gb300"


class _Writer:
    """One background thread that runs queued file writes in order."""

    def __init__(self):
        self.q: queue.Queue = queue.Queue(maxsize=64)
        self.error: BaseException | None = None
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _run(self):
        while True:
            job = self.q.get()
            if job is None:
                return
            if self.error is None:
                try:
                    job()
                except BaseException as e:  # reported on close()
                    self.error = e

    def submit(self, job) -> None:
        if self.error is not None:
            raise RuntimeError("observer write failed") from self.error
        self.q.put(job)

    def close(self) -> None:
        self.q.put(None)
        self.t.join()
        if self.error is not None:
            raise RuntimeError("observer write failed") from self.error


def _record(fh, payload: bytes) -> None:
    n = struct.pack("<i", len(payload))
    fh.write(n + payload + n)


def write_dcd_header(fh, n_particles: int, total_frames: int, save_interval: int, total_step: int,
                     delta_t: float, use_periodic: bool) -> None:
    """The three header records of src/Observer.cpp:120-188."""
    first = (b"CORD" + struct.pack("<9i", total_frames, 0, save_interval, total_step, 0, 0, 0, 0, 0)
             + struct.pack("<f", delta_t) + struct.pack("<i", int(use_periodic)) + struct.pack("<8i", *([0] * 8))
             + struct.pack("<i", 24))
    _record(fh, first)
    _record(fh, struct.pack("<i", 1) + DCD_TITLE.ljust(80, b"\0")[:80])
    _record(fh, struct.pack("<i", n_particles))


def write_dcd_frame(fh, xyz_angstrom: np.ndarray, box_angstrom=None) -> None:
    """Optional unit cell, then the x, y, z float32 records."""
    if box_angstrom is not None:
        a, b, c = (float(v) for v in box_angstrom)
        _record(fh, struct.pack("<6d", a, 90.0, b, 90.0, 90.0, c))
    xyz = np.asarray(xyz_angstrom, np.float32)
    for k in range(3):
        _record(fh, np.ascontiguousarray(xyz[:, k]).tobytes())


def read_dcd(path, unitcells: bool | None = None) -> dict:
    """Read a DCD written by ``DCDObserver`` (or the reference).  The
    velocity file's header carries the same unit-cell flag as the position
    file but its frames have no unit-cell record: pass ``unitcells=False``
    to read a periodic system's velocity file."""
    data = Path(path).read_bytes()
    pos = 0

    def rec():
        nonlocal pos
        (n,) = struct.unpack_from("<i", data, pos)
        payload = data[pos + 4: pos + 4 + n]
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        if m != n:
            raise ValueError("corrupt DCD record")
        pos += 8 + n
        return payload

    first = rec()
    if first[:4] != b"CORD":
        raise ValueError("not a DCD file")
    ints = struct.unpack_from("<9i", first, 4)
    (delta_t,) = struct.unpack_from("<f", first, 40)
    (has_cell,) = struct.unpack_from("<i", first, 44)
    cell_records = bool(has_cell) if unitcells is None else bool(unitcells)
    (version,) = struct.unpack_from("<i", first, 80)
    title = rec()
    (natoms,) = struct.unpack("<i", rec())
    frames, cells = [], []
    while pos < len(data):
        if cell_records:
            cells.append(struct.unpack("<6d", rec()))
        xyz = [np.frombuffer(rec(), np.float32) for _ in range(3)]
        frames.append(np.stack(xyz, 1))
    return {"total_frames": ints[0], "first": ints[1], "save_interval": ints[2], "total_step": ints[3],
            "delta_t": delta_t, "has_unitcell": bool(has_cell), "version": version,
            "title": title[4:].rstrip(b"\0"), "n_particles": natoms,
            "frames": np.array(frames), "unitcells": np.array(cells) if cells else None}


class ObserverBase:
    def initialize(self, context, writer: _Writer) -> None:  # pragma: no cover - interface
        raise NotImplementedError

    def output(self, step: int, context, writer: _Writer) -> None:  # pragma: no cover
        raise NotImplementedError

    def finalize(self, writer: _Writer) -> None:
        pass


class EnergyObserver(ObserverBase):
    """``<prefix>.ene`` in kcal/mol (src/Observer.cpp:302-347)."""

    def __init__(self, file_prefix: str, system):
        self.path = Path(str(file_prefix) + ".ene")
        names = system.group_names()
        # the reference iterates a std::map<name, group>: name order
        self.columns = sorted((name, g) for g, name in enumerate(names))

    def header(self) -> str:
        cols = "".join(f" {name:>24}" for name, _ in self.columns)
        return f"# unit of energy : kcal/mol\n# timestep{cols} kinetic_energy\n"

    def line(self, step: int, group_kj: np.ndarray, kinetic_kj: float) -> str:
        vals = "".join(f" {group_kj[g] * KCAL_PER_KJ:>24.6f}" for _, g in self.columns)
        return f"{step:<10d}{vals} {kinetic_kj * KCAL_PER_KJ:>14.6f}\n"

    def initialize(self, context, writer: _Writer) -> None:
        text = self.header()
        writer.submit(lambda: self.path.write_text(text))

    def output(self, step: int, context, writer: _Writer) -> None:
        e = context.getGroupEnergies()
        ke = context.getKineticEnergy()
        text = self.line(step, e, ke)

        def job():
            with open(self.path, "a") as fh:
                fh.write(text)
        writer.submit(job)


class DCDObserver(ObserverBase):
    """``<prefix>_position.dcd`` and ``<prefix>_velocity.dcd``
    (src/Observer.cpp:66-300).  ``delta_t`` is the input file's step in
    cafetime, as the reference writes it; ``box_nm`` is the periodic box
    (cuboid) or None."""

    def __init__(self, file_prefix: str, total_step: int, save_interval: int, delta_t: float,
                 use_periodic: bool, box_nm=None):
        self.pos_path = Path(str(file_prefix) + "_position.dcd")
        self.vel_path = Path(str(file_prefix) + "_velocity.dcd")
        self.total_step, self.save_interval = int(total_step), int(save_interval)
        self.delta_t, self.use_periodic = float(delta_t), bool(use_periodic)
        if self.use_periodic and box_nm is None:
            raise ValueError("a periodic DCD needs the box")
        self.box = None if box_nm is None else np.asarray(box_nm, float) * ANGSTROM_PER_NM

    def initialize(self, context, writer: _Writer) -> None:
        n = context.n
        frames = self.total_step // self.save_interval

        def job():
            for p in (self.pos_path, self.vel_path):
                with open(p, "wb") as fh:
                    write_dcd_header(fh, n, frames, self.save_interval, self.total_step, self.delta_t,
                                     self.use_periodic)
        writer.submit(job)

    def output(self, step: int, context, writer: _Writer) -> None:
        x = context.getPositions() * ANGSTROM_PER_NM
        v = context.getVelocities() * ANGSTROM_PER_NM * CAFETIME_PS
        box = self.box if self.use_periodic else None

        def job():
            with open(self.pos_path, "ab") as fh:
                write_dcd_frame(fh, x, box)
            with open(self.vel_path, "ab") as fh:
                write_dcd_frame(fh, v)
        writer.submit(job)


class PDBObserver(ObserverBase):
    """``<prefix>.pdb`` MODEL frames (src/Observer.cpp:7-63)."""

    def __init__(self, file_prefix: str, names):
        self.path = Path(str(file_prefix) + ".pdb")
        self.names = [("UNK" if nm is None else str(nm)) for nm in names]

    def initialize(self, context, writer: _Writer) -> None:
        writer.submit(lambda: self.path.write_text(""))

    def output(self, step: int, context, writer: _Writer) -> None:
        x = context.getPositions() * ANGSTROM_PER_NM

        def job():
            lines = [f"MODEL     {step}\n"]
            for i, (p, nm) in enumerate(zip(x, self.names)):
                lines.append(f"ATOM  {i + 1:>5}   CA {nm:>3}     1    {p[0]:8.3f}{p[1]:8.3f}{p[2]:8.3f}"
                             "  1.00  0.00\n")
            lines.append("ENDMDL\n")
            with open(self.path, "a") as fh:
                fh.write("".join(lines))
        writer.submit(job)


class Simulator:
    """The reference's run loop (src/Simulator.cpp:37-76) on a Context:
    ``initialize`` sets the positions and, when asked, minimises the energy
    first; ``run`` lets each observer record the state every ``save_step``
    steps, then advances the integrator ``save_step`` steps; observer output
    is written by a background thread."""

    def __init__(self, context, total_step: int, save_step: int, observers=(),
                 energy_minimization: bool = False):
        if save_step <= 0:
            raise ValueError("save_step must be positive")
        self.context = context
        self.total_step, self.save_step = int(total_step), int(save_step)
        self.observers = list(observers)
        self.energy_minimization = bool(energy_minimization)

    def initialize(self, positions) -> None:
        self.context.setPositions(positions)
        if self.energy_minimization:
            from .engine import LocalEnergyMinimizer
            LocalEnergyMinimizer.minimize(self.context)

    def run(self) -> None:
        writer = _Writer()
        try:
            for ob in self.observers:
                ob.initialize(self.context, writer)
            for frame in range(self.total_step // self.save_step):
                for ob in self.observers:
                    ob.output(frame * self.save_step, self.context, writer)
                self.context.step(self.save_step)
            for ob in self.observers:
                ob.finalize(writer)
        finally:
            writer.close()
