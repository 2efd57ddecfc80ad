"""Continuous-batching request loop over the batched engine.

Requests (one coarse-grained system each, with its own temperature, seed
and step count) arrive over time.  The loop admits waiting requests while
their device footprint (``ocm_batch_footprint``: parameters, lists and bead
state) fits the device-memory budget and the batch has a free slot and bead
capacity, advances every resident system with one launch per chunk,
retires finished systems (freeing their memory for the next admissions)
and records each request's completion latency.  Admission happens while a
chunk runs and every other system stays resident on the device, so new
work overlaps with work already running.

Launches are balanced: the largest resident system advances
``chunk_steps`` steps per launch and smaller ones proportionally more, so
one large request does not hold every small one to its pace (each
trajectory is independent of how its steps are split into launches).  A
system that blows up is retired as failed and its request completes with
``failed = True``.  A request whose ``cancelled`` flag the client sets
leaves the queue, or its slot, at the next pass of the loop.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import OCMError
from .engine import Batch
from .forcefield import System


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the stream starts
    system: System
    positions: np.ndarray
    temperature: float
    n_steps: int
    seed: int
    friction: float = 0.1
    step_size: float = 0.01
    # filled in by the server
    admitted_at: float = math.nan
    finished_at: float = math.nan
    result: np.ndarray | None = None
    failed: bool = False
    footprint: int = -1     # device bytes in a batch (computed at the first admission attempt)
    # set by the client (any thread) to withdraw the request: a waiting one
    # is dropped, a resident one retired at the next pass of the loop; it
    # completes with the steps it did and no result
    cancelled: bool = False

    @property
    def beads(self) -> int:
        return self.system.n

    @property
    def latency(self) -> float:
        return self.finished_at - self.arrival


@dataclass
class ServeStats:
    requests: int
    wall_s: float
    bead_steps: float
    latencies_s: list = field(default_factory=list)
    chunks: int = 0
    max_resident: int = 0
    hbm_budget_bytes: int | None = None
    peak_resident_bytes: int = 0
    waits_for_memory: int = 0   # admission attempts deferred by the budget
    failed: int = 0
    cancelled: int = 0

    def summary(self) -> dict:
        lat = np.array(self.latencies_s)
        return {"requests": self.requests, "wall_s": self.wall_s,
                "bead_steps_per_s": self.bead_steps / self.wall_s if self.wall_s > 0 else None,
                "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
                "chunks": self.chunks, "max_resident": self.max_resident,
                "hbm_budget_bytes": self.hbm_budget_bytes, "peak_resident_bytes": self.peak_resident_bytes,
                "waits_for_memory": self.waits_for_memory, "failed": self.failed,
                "cancelled": self.cancelled}


class Server:
    """Owns a Batch and runs a request stream through it.

    ``hbm_budget_bytes``: device memory the resident systems may occupy
    together (their footprints); None = only the batch's own capacity."""

    def __init__(self, max_systems: int, max_total_beads: int, max_beads_per_system: int,
                 chunk_steps: int = 200, device: int = 0, keep_results: bool = False,
                 hbm_budget_bytes: int | None = None, balanced: bool = True, batch=None):
        """``batch``: an existing object with Batch's admit / run / finished /
        status / positions / steps_done / retire / footprint calls to serve
        through (default: a new Batch of the given capacity)."""
        self.batch = batch if batch is not None else Batch(max_systems, max_total_beads, max_beads_per_system,
                                                           device=device)
        self.batch.set_balanced(balanced)
        self.chunk_steps = chunk_steps
        self.max_systems = max_systems
        self.keep_results = keep_results
        self.hbm_budget_bytes = hbm_budget_bytes

    def serve(self, requests: list[Request], realtime: bool = True) -> ServeStats:
        """Run the stream.  With realtime=True requests become visible at
        their arrival times on the wall clock; otherwise all arrive at once."""
        queue = sorted(requests, key=lambda r: r.arrival)
        waiting: list[Request] = []
        resident: dict[int, Request] = {}
        done = 0
        nxt = 0
        stats = ServeStats(requests=len(queue), wall_s=0.0, bead_steps=0.0,
                           hbm_budget_bytes=self.hbm_budget_bytes)
        footprint: dict[int, int] = {}   # slot -> device bytes
        resident_bytes = 0
        t0 = time.perf_counter()
        while done < len(queue):
            now = time.perf_counter() - t0 if realtime else math.inf
            while nxt < len(queue) and queue[nxt].arrival <= now:
                waiting.append(queue[nxt])
                nxt += 1
            # withdrawn requests: waiting ones leave the queue, resident ones
            # their slots
            for r in [r for r in waiting if r.cancelled]:
                waiting.remove(r)
                self._complete(r, t0, realtime, stats, steps=0)
                done += 1
            for slot in [k for k, r in resident.items() if r.cancelled]:
                r = resident.pop(slot)
                steps = self.batch.steps_done(slot)
                self.batch.retire(slot)
                resident_bytes -= footprint.pop(slot)
                self._complete(r, t0, realtime, stats, steps=steps)
                done += 1
            if done == len(queue):
                break
            ran = False
            if resident:
                # launch the chunk first: the admissions below (host-side
                # compile + uploads on the copy stream) overlap with it
                self.batch.run(self.chunk_steps, sync=False)
                stats.chunks += 1
                ran = True
            while waiting and len(resident) < self.max_systems:
                r = waiting[0]
                if r.footprint < 0:
                    r.footprint = self.batch.footprint(r.system)
                need = r.footprint
                if self.hbm_budget_bytes is not None and resident_bytes + need > self.hbm_budget_bytes:
                    if not resident:
                        raise OCMError(3, f"request {r.rid} needs {need} bytes, more than the whole "
                                          f"budget of {self.hbm_budget_bytes}")
                    stats.waits_for_memory += 1
                    break  # wait for a retirement to free memory
                try:
                    slot = self.batch.admit(r.system, r.positions, temperature=r.temperature,
                                            friction=r.friction, step_size=r.step_size,
                                            seed=r.seed, n_steps=r.n_steps)
                except OCMError as e:
                    if e.code == 3:  # no capacity now: retry after a retirement
                        break
                    raise
                r.admitted_at = time.perf_counter() - t0
                resident[slot] = r
                footprint[slot] = need
                resident_bytes += need
                waiting.pop(0)
            stats.max_resident = max(stats.max_resident, len(resident))
            stats.peak_resident_bytes = max(stats.peak_resident_bytes, resident_bytes)
            if not ran:
                if not resident and nxt < len(queue) and realtime:
                    time.sleep(max(0.0, queue[nxt].arrival - (time.perf_counter() - t0)))
                continue
            for slot in self.batch.finished():
                if slot not in resident:
                    continue
                r = resident.pop(slot)
                r.failed = self.batch.status(slot) != 0
                if self.keep_results:
                    r.result = self.batch.positions(slot)
                steps = self.batch.steps_done(slot)
                self.batch.retire(slot)
                resident_bytes -= footprint.pop(slot)
                self._complete(r, t0, realtime, stats, steps=steps)
                done += 1
        stats.wall_s = time.perf_counter() - t0
        return stats

    @staticmethod
    def _complete(r: Request, t0: float, realtime: bool, stats: ServeStats, steps: int) -> None:
        r.finished_at = time.perf_counter() - t0
        stats.latencies_s.append(r.latency if realtime else r.finished_at)
        stats.bead_steps += r.beads * steps
        stats.failed += int(r.failed)
        stats.cancelled += int(r.cancelled)


def poisson_arrivals(n: int, rate_per_s: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, n))


def log_uniform_int(rng: np.random.Generator, lo: float, hi: float, n: int) -> np.ndarray:
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), n))).astype(np.int64)
