"""The continuous-batching loop's host logic with a stand-in batch (no GPU):
admission against slot, bead and device-memory limits, waits for
retirements, completion records, failed and cancelled requests."""
import numpy as np
import pytest

from opencafemol_gb300 import serving
from opencafemol_gb300._lib import OCMError


class _System:
    def __init__(self, n):
        self.n = n


class _FakeBatch:
    """Batch's calls as the server uses them: every resident system
    advances by the launch's steps until its target; systems whose seed is
    in ``blow_up`` stop after their first launch with status 7."""

    def __init__(self, max_systems, max_beads, blow_up=()):
        self.max_systems, self.max_beads, self.blow_up = max_systems, max_beads, set(blow_up)
        self.slots = {}
        self.launches = 0
        self.balanced = None

    def set_balanced(self, on):
        self.balanced = on

    @staticmethod
    def footprint(system):
        return 1000 * system.n

    def admit(self, system, positions, temperature, friction, step_size, seed, n_steps):
        used = sum(v["n"] for v in self.slots.values())
        if len(self.slots) >= self.max_systems or used + system.n > self.max_beads:
            raise OCMError(3, "no capacity")
        slot = min(set(range(self.max_systems)) - set(self.slots))
        self.slots[slot] = {"n": system.n, "target": n_steps, "done": 0, "status": 0, "seed": seed}
        return slot

    def run(self, k, sync=False):
        self.launches += 1
        for v in self.slots.values():
            if v["status"] or v["done"] >= v["target"]:
                continue
            if v["seed"] in self.blow_up:
                v["done"] += 1
                v["status"] = 7
            else:
                v["done"] = min(v["target"], v["done"] + k)

    def finished(self):
        return [s for s, v in self.slots.items() if v["status"] or v["done"] >= v["target"]]

    def status(self, slot):
        return self.slots[slot]["status"]

    def positions(self, slot):
        return np.full((self.slots[slot]["n"], 3), float(slot))

    def steps_done(self, slot):
        return self.slots[slot]["done"]

    def retire(self, slot):
        del self.slots[slot]


def _requests(sizes, steps, seeds=None):
    seeds = seeds if seeds is not None else list(range(len(sizes)))
    return [serving.Request(rid=k, arrival=0.0, system=_System(n), positions=np.zeros((n, 3)),
                            temperature=300.0, n_steps=s, seed=seeds[k])
            for k, (n, s) in enumerate(zip(sizes, steps))]


def test_every_request_completes_with_its_work():
    sizes, steps = [50, 300, 120, 800, 60], [400, 150, 1000, 90, 10]
    fake = _FakeBatch(max_systems=2, max_beads=900)
    server = serving.Server(2, 900, 800, chunk_steps=100, keep_results=True, batch=fake)
    reqs = _requests(sizes, steps)
    st = server.serve(reqs, realtime=False)
    assert fake.balanced is True
    assert st.requests == 5 and len(st.latencies_s) == 5 and st.failed == 0
    assert st.max_resident <= 2
    assert st.bead_steps == sum(n * s for n, s in zip(sizes, steps))
    assert all(r.result is not None and r.result.shape == (r.beads, 3) for r in reqs)
    assert not fake.slots  # everything retired


def test_device_memory_budget_defers_admissions():
    sizes, steps = [200, 200, 200, 200], [300, 300, 300, 300]
    fake = _FakeBatch(max_systems=8, max_beads=10 ** 6)
    budget = 2 * 200 * 1000  # two systems' footprints
    server = serving.Server(8, 10 ** 6, 800, chunk_steps=100, hbm_budget_bytes=budget, batch=fake)
    st = server.serve(_requests(sizes, steps), realtime=False)
    assert len(st.latencies_s) == 4
    assert st.peak_resident_bytes == budget and st.max_resident == 2
    assert st.waits_for_memory > 0


def test_request_larger_than_the_budget_is_refused():
    fake = _FakeBatch(max_systems=4, max_beads=10 ** 6)
    server = serving.Server(4, 10 ** 6, 800, hbm_budget_bytes=50 * 1000, batch=fake)
    with pytest.raises(OCMError) as ei:
        server.serve(_requests([100], [10]), realtime=False)
    assert ei.value.code == 3


def test_blown_up_request_completes_as_failed():
    fake = _FakeBatch(max_systems=4, max_beads=10 ** 6, blow_up={11})
    server = serving.Server(4, 10 ** 6, 800, chunk_steps=50, batch=fake)
    reqs = _requests([40, 70, 90], [200, 200, 200], seeds=[10, 11, 12])
    st = server.serve(reqs, realtime=False)
    assert st.failed == 1 and [r.failed for r in reqs] == [False, True, False]
    # the failed request counts the one step it did
    assert st.bead_steps == 40 * 200 + 70 * 1 + 90 * 200


def test_capacity_waits_then_admits_after_retirement():
    # bead capacity for one large system at a time
    fake = _FakeBatch(max_systems=4, max_beads=1000)
    server = serving.Server(4, 1000, 800, chunk_steps=100, batch=fake)
    st = server.serve(_requests([800, 700, 600], [100, 100, 100]), realtime=False)
    assert len(st.latencies_s) == 3 and st.max_resident == 1
    assert fake.launches >= 3


def test_cancelled_requests_leave_queue_and_slot():
    """A resident request cancelled by its client gives up its slot at the
    next pass (completing with the steps it did, no result); a waiting one
    never gets admitted; the others complete."""
    reqs = _requests([100, 200, 300, 400], [1000, 1000, 1000, 1000])

    class _Client(_FakeBatch):
        def run(self, k, sync=False):
            super().run(k, sync)
            if self.launches == 2:
                reqs[0].cancelled = True  # resident by now
                reqs[3].cancelled = True  # still waiting (capacity two)

    fake = _Client(max_systems=2, max_beads=10 ** 6)
    server = serving.Server(2, 10 ** 6, 800, chunk_steps=100, keep_results=True, batch=fake)
    st = server.serve(reqs, realtime=False)
    assert st.cancelled == 2 and len(st.latencies_s) == 4 and st.failed == 0
    assert reqs[0].result is None and reqs[3].result is None
    assert reqs[1].result is not None and reqs[2].result is not None
    # request 0 ran two launches; request 3 never ran
    assert st.bead_steps == 100 * 200 + 200 * 1000 + 300 * 1000
    assert not fake.slots
