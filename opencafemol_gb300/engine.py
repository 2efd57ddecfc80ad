"""Device engines behind the C ABI.

``Context`` is the plain single-system path: the part of an OpenMM
``Context`` + ``LangevinIntegrator`` that the reference's ``Simulator``
drives (src/Simulator.cpp:17-76).  ``Batch`` is the batched / served path:
many independent systems advanced by one persistent kernel per chunk.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import OCM_MAX_GROUPS, ContextStats, OCMError, as_f64, check, dptr, i64ptr, lib
from .forcefield import LangevinIntegrator, System

__all__ = ["Context", "Batch", "ALL_GROUPS", "LocalEnergyMinimizer"]

ALL_GROUPS = 0xFFFFFFFF


class Context:
    """OpenMM's Context + LangevinIntegrator as the reference's Simulator
    drives them.  ``engine`` picks the kernels of ``step``: "auto" (a
    non-periodic system of at most 512 beads as a one-system persistent
    launch of the batched kernel, anything else on the cluster-pair tiles),
    "tiles" or "one_system"."""

    ENGINES = {"auto": 0, "tiles": 1, "one_system": 2}

    def __init__(self, system: System, integrator: LangevinIntegrator, device: int = 0, engine: str = "auto"):
        self.system = system  # keeps the system alive
        self.n = system.n
        h = C.c_void_p()
        check(lib.ocm_context_create(system.handle, integrator.temperature, integrator.friction,
                                     integrator.step_size, integrator.seed, int(device), C.byref(h)))
        self._h = h
        if engine != "auto":
            self.set_engine(engine)

    def set_engine(self, engine: str) -> None:
        check(lib.ocm_context_set_engine(self._h, Context.ENGINES[engine]))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.ocm_context_destroy(h)
            self._h = None

    def setPositions(self, xyz) -> None:
        a = as_f64(xyz).reshape(self.n, 3)
        check(lib.ocm_context_set_positions(self._h, dptr(a)))

    def getPositions(self) -> np.ndarray:
        a = np.zeros((self.n, 3))
        check(lib.ocm_context_get_positions(self._h, dptr(a)))
        return a

    def setVelocities(self, v) -> None:
        a = as_f64(v).reshape(self.n, 3)
        check(lib.ocm_context_set_velocities(self._h, dptr(a)))

    def getVelocities(self) -> np.ndarray:
        a = np.zeros((self.n, 3))
        check(lib.ocm_context_get_velocities(self._h, dptr(a)))
        return a

    def setVelocitiesToTemperature(self, temperature: float, seed: int) -> None:
        check(lib.ocm_context_set_velocities_to_temperature(self._h, float(temperature), int(seed)))

    def getState(self, forces: bool = True, energy: bool = True, groups: int = ALL_GROUPS):
        """Return (forces [n,3] kJ/mol/nm or None, potential energy kJ/mol or None)."""
        f = np.zeros((self.n, 3)) if forces else None
        e = C.c_double()
        check(lib.ocm_context_get_state(self._h, C.c_uint32(groups), dptr(f),
                                        C.byref(e) if energy else None))
        return f, (e.value if energy else None)

    def getGroupEnergies(self) -> np.ndarray:
        e = np.zeros(OCM_MAX_GROUPS)
        check(lib.ocm_context_get_group_energies(self._h, dptr(e)))
        return e

    def getKineticEnergy(self) -> float:
        e = C.c_double()
        check(lib.ocm_context_get_kinetic_energy(self._h, C.byref(e)))
        return e.value

    def step(self, steps: int) -> None:
        check(lib.ocm_context_step(self._h, int(steps)))

    def stats(self) -> dict:
        s = ContextStats()
        check(lib.ocm_context_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ContextStats._fields_}

    def set_list_options(self, rebuild_interval: int = 0, skin: float = 0.0) -> None:
        check(lib.ocm_context_set_list_options(self._h, int(rebuild_interval), float(skin)))

    def list_pairs(self) -> np.ndarray:
        n = C.c_int64()
        cap = max(1024, self.n * 64)
        while True:
            out = np.zeros((cap, 2), np.int64)
            try:
                check(lib.ocm_context_list_pairs(self._h, i64ptr(out), cap, C.byref(n)))
                return out[: n.value].copy()
            except OCMError:
                if n.value > cap:
                    cap = n.value
                    continue
                raise

    def cluster_order(self) -> np.ndarray:
        """Bead index of every cluster slot (-1 for padding slots)."""
        n = C.c_int64()
        cap = self.n + 64
        while True:
            out = np.zeros(cap, np.int64)
            try:
                check(lib.ocm_context_cluster_order(self._h, i64ptr(out), cap, C.byref(n)))
                return out[: n.value].copy()
            except OCMError:
                if n.value > cap:
                    cap = n.value
                    continue
                raise


class LocalEnergyMinimizer:
    """OpenMM's ``LocalEnergyMinimizer.minimize(context, tolerance,
    maxIterations)`` as the reference's Simulator calls it before a run
    (src/Simulator.cpp:41-46): L-BFGS on the potential energy until the RMS
    of all force components is at most ``tolerance`` kJ/mol/nm, or
    ``maxIterations`` iterations (0: no limit).  Returns the iterations."""

    REASONS = ("converged", "iteration limit", "stagnated at the FP32 force floor", "line search failed")

    @staticmethod
    def minimize(context: Context, tolerance: float = 10.0, maxIterations: int = 0) -> int:
        it = C.c_int64()
        check(lib.ocm_context_minimize(context._h, float(tolerance), int(maxIterations), C.byref(it)))
        return it.value

    @staticmethod
    def report(context: Context) -> dict:
        """Why the last minimisation of ``context`` stopped, and the RMS
        force it reached (the tolerance may be below the FP32 force floor)."""
        r, rms = C.c_int32(), C.c_double()
        check(lib.ocm_context_minimize_report(context._h, C.byref(r), C.byref(rms)))
        return {"reason": LocalEnergyMinimizer.REASONS[r.value], "code": r.value, "rms_force": rms.value}


class Batch:
    """Device-resident ensemble of independent systems."""

    def __init__(self, max_systems: int, max_total_beads: int, max_beads_per_system: int,
                 device: int = 0):
        h = C.c_void_p()
        check(lib.ocm_batch_create(int(device), int(max_systems), int(max_total_beads),
                                   int(max_beads_per_system), C.byref(h)))
        self._h = h
        self._n: dict[int, int] = {}
        self._systems: dict[int, System] = {}
        self._sizes = np.zeros(int(max_systems), np.int64)  # beads per slot (0: free)

    def _total(self, sl: np.ndarray) -> int:
        """Beads of the slots in ``sl`` (out-of-range slots count 0: the C
        call refuses them)."""
        if sl.size == 0 or sl.min() < 0 or sl.max() >= self._sizes.size:
            return 0
        return int(self._sizes[sl].sum())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.ocm_batch_destroy(h)
            self._h = None

    @staticmethod
    def footprint(system: System) -> int:
        return system.footprint()

    def admit(self, system: System, positions, velocities=None, temperature: float = 300.0,
              friction: float = 0.1, step_size: float = 0.01, seed: int = 0, n_steps: int = 0,
              steps_done: int = 0) -> int:
        """Admit a system into a free slot.  ``steps_done`` > 0 resumes a
        trajectory that already ran that many of its ``n_steps`` steps
        (velocities required): the Langevin noise continues from that step,
        so the positions and velocities read back from the slot it left
        give the uninterrupted trajectory."""
        pos = as_f64(positions).reshape(system.n, 3)
        vel = None if velocities is None else as_f64(velocities).reshape(system.n, 3)
        slot = C.c_int64()
        if steps_done:
            if vel is None:
                raise ValueError("resuming a trajectory needs its velocities")
            check(lib.ocm_batch_admit_resume(self._h, system.handle, dptr(pos), dptr(vel), float(temperature),
                                             float(friction), float(step_size), int(seed), int(n_steps),
                                             int(steps_done), C.byref(slot)))
        else:
            check(lib.ocm_batch_admit(self._h, system.handle, dptr(pos), dptr(vel), float(temperature),
                                      float(friction), float(step_size), int(seed), int(n_steps),
                                      C.byref(slot)))
        self._n[slot.value] = system.n
        self._sizes[slot.value] = system.n
        self._systems[slot.value] = system
        return slot.value

    def run(self, steps_per_launch: int, sync: bool = False) -> None:
        check(lib.ocm_batch_run(self._h, int(steps_per_launch), int(sync)))

    def status(self, slot: int) -> int:
        """0, or 7 (OCMError code NONFINITE) if the slot's system blew up and
        stopped advancing."""
        st = C.c_int32()
        check(lib.ocm_batch_slot_status(self._h, int(slot), C.byref(st)))
        return st.value

    def finished(self) -> list[int]:
        n = C.c_int64()
        cap = max(1, len(self._n))
        out = np.zeros(cap, np.int64)
        check(lib.ocm_batch_finished(self._h, i64ptr(out), cap, C.byref(n)))
        return [int(v) for v in out[: min(n.value, cap)]]

    def positions(self, slot: int) -> np.ndarray:
        a = np.zeros((self._n[slot], 3))
        check(lib.ocm_batch_get_positions(self._h, int(slot), dptr(a)))
        return a

    def velocities(self, slot: int) -> np.ndarray:
        a = np.zeros((self._n[slot], 3))
        check(lib.ocm_batch_get_velocities(self._h, int(slot), dptr(a)))
        return a

    def set_positions_many(self, slots, xyz, velocities=None) -> None:
        """Positions (and velocities) of many slots, beads back to back."""
        sl = np.ascontiguousarray(slots, np.int64)
        x = as_f64(xyz)
        v = None if velocities is None else as_f64(velocities)
        total = self._total(sl)
        if x.size != 3 * total or (v is not None and v.size != 3 * total):
            raise ValueError(f"positions (and velocities) must hold {total} x 3 values for these slots")
        check(lib.ocm_batch_set_positions_many(self._h, len(sl), i64ptr(sl), dptr(x), dptr(v)))

    @staticmethod
    def _out_buffer(out, total: int) -> np.ndarray:
        """The caller's output array, or a new one; the C call writes
        total x 3 doubles into it, so anything else is refused."""
        if out is None:
            return np.zeros((total, 3))
        if (not isinstance(out, np.ndarray) or out.dtype != np.float64 or out.shape != (total, 3)
                or not out.flags.c_contiguous or not out.flags.writeable):
            raise ValueError(f"out must be a writeable C-contiguous float64 array of shape ({total}, 3)")
        return out

    def get_positions_many(self, slots, out=None) -> np.ndarray:
        sl = np.ascontiguousarray(slots, np.int64)
        total = self._total(sl)
        out = self._out_buffer(out, total)
        check(lib.ocm_batch_get_positions_many(self._h, len(sl), i64ptr(sl), dptr(out)))
        return out

    def get_positions_many_noalloc(self, slots, out=None) -> np.ndarray:
        """``get_positions_many`` through fixed per-device scratch (no device
        allocation; at most 131072 beads and 2048 slots per call)."""
        sl = np.ascontiguousarray(slots, np.int64)
        total = self._total(sl)
        out = self._out_buffer(out, total)
        check(lib.ocm_batch_get_positions_many_noalloc(self._h, len(sl), i64ptr(sl), dptr(out)))
        return out

    def steps_done(self, slot: int) -> int:
        s = C.c_int64()
        check(lib.ocm_batch_steps_done(self._h, int(slot), C.byref(s)))
        return s.value

    def state(self, slot: int, groups: int = ALL_GROUPS):
        f = np.zeros((self._n[slot], 3))
        e = np.zeros(OCM_MAX_GROUPS)
        check(lib.ocm_batch_get_state(self._h, int(slot), C.c_uint32(groups), dptr(f), dptr(e)))
        return f, e

    def retire(self, slot: int) -> None:
        check(lib.ocm_batch_retire(self._h, int(slot)))
        self._n.pop(slot, None)
        self._sizes[slot] = 0
        self._systems.pop(slot, None)

    def active(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        check(lib.ocm_batch_active(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_threads(self, threads_per_cta: int) -> None:
        check(lib.ocm_batch_set_threads(self._h, int(threads_per_cta)))

    def set_list_smem(self, kib: int) -> None:
        check(lib.ocm_batch_set_list_smem(self._h, int(kib)))

    def set_split(self, beads: int) -> None:
        """Tuning knob: CTAs split into two groups once their systems have
        at most ``beads`` beads (0: never)."""
        check(lib.ocm_batch_set_split(self._h, int(beads)))

    def set_balanced(self, on: bool = True) -> None:
        """Balanced launches: the costliest system does the launch's steps,
        smaller ones proportionally more (for a serving loop)."""
        check(lib.ocm_batch_set_balanced(self._h, int(bool(on))))

    # (threads per CTA, list shared memory KiB, split beads); -1 KiB = no cap
    DEFAULT_TUNE_CANDIDATES = ((512, 96, 512), (512, -1, 512), (512, 96, 384), (1024, 96, 512),
                               (1024, -1, 512), (512, 96, 0), (1024, 96, 0), (256, 96, 384))

    def autotune(self, steps_per_trial: int = 50, candidates=DEFAULT_TUNE_CANDIDATES,
                 rounds: int = 2) -> dict:
        """Pick the launch shape (threads per CTA, list shared memory in KiB,
        split size) for the systems resident now.  A candidate of two
        entries keeps split 0.

        In each of ``rounds`` rounds every candidate runs two real launches
        of ``steps_per_trial`` steps (the first absorbs the set-up of that
        shape); the second is timed with CUDA events.  The rounds interleave
        the candidates, so a transient of the systems' cost while they relax
        spreads over every candidate instead of falling on the first ones
        (warm up before tuning, as the benchmark does); the shape with the
        smallest mean time is kept.  Trajectories do not depend on the
        shape, so the trials are ordinary simulation progress: the resident
        systems advance by 2 * rounds * steps_per_trial steps per candidate
        (systems with fewer steps left finish early)."""
        cands = [(c[0], c[1], c[2] if len(c) > 2 else 0) for c in candidates]
        times = [[] for _ in cands]
        for _ in range(max(1, rounds)):
            for k, (th, kib, split) in enumerate(cands):
                self.set_threads(th)
                self.set_list_smem(kib)
                self.set_split(split)
                self.run(steps_per_trial, sync=True)
                self.run(steps_per_trial, sync=True)
                times[k].append(self.last_run_ms())
        trials = [(sum(t) / len(t), th, kib, split) for t, (th, kib, split) in zip(times, cands)]
        ms, th, kib, split = min(trials)
        self.set_threads(th)
        self.set_list_smem(kib)
        self.set_split(split)
        return {"threads": th, "list_smem_kib": kib, "split_beads": split, "ms_per_launch": ms,
                "trials": [{"threads": t, "list_smem_kib": k, "split_beads": sp, "ms": m}
                           for m, t, k, sp in trials]}

    def threads(self) -> int:
        t = C.c_int32()
        check(lib.ocm_batch_get_threads(self._h, C.byref(t)))
        return t.value

    def slot_stats(self, slot: int) -> dict:
        b, c = C.c_int32(), C.c_int32()
        check(lib.ocm_batch_slot_stats(self._h, int(slot), C.byref(b), C.byref(c)))
        return {"list_builds": b.value, "list_capacity": c.value}

    def last_run_ms(self) -> float:
        ms = C.c_double()
        check(lib.ocm_batch_last_run_ms(self._h, C.byref(ms)))
        return ms.value
