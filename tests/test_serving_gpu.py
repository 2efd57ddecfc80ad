"""Continuous batching: requests admitted while others run, capacity freed by
retirements, and every result identical to the same request run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(n, seed=0):
    from opencafemol_gb300 import serving, synth
    rng = np.random.default_rng(seed)
    sizes = serving.log_uniform_int(rng, 30, 700, n)
    steps = serving.log_uniform_int(rng, 50, 400, n)
    temps = rng.uniform(280, 360, n)
    reqs = []
    for k in range(n):
        spec = synth.go_protein(int(sizes[k]), 7000 + k, temperature=float(temps[k]))
        reqs.append(serving.Request(rid=k, arrival=0.001 * k, system=synth.build_system(spec),
                                    positions=spec.pos, temperature=float(temps[k]),
                                    n_steps=int(steps[k]), seed=100 + k))
    return reqs


def test_stream_completes_and_matches_alone(gpu):
    from opencafemol_gb300 import serving
    reqs = _requests(14)
    # capacity for only a few systems at a time forces admission waits
    server = serving.Server(max_systems=4, max_total_beads=1600, max_beads_per_system=700,
                            chunk_steps=37, keep_results=True)
    stats = server.serve(reqs, realtime=False)
    assert stats.requests == 14 and len(stats.latencies_s) == 14
    assert stats.max_resident <= 4
    for r in reqs[:5]:
        alone = gpu.Batch(max_systems=1, max_total_beads=800, max_beads_per_system=700)
        slot = alone.admit(r.system, r.positions, temperature=r.temperature, seed=r.seed,
                           n_steps=r.n_steps)
        while alone.finished() != [slot]:
            alone.run(50)
        assert np.array_equal(alone.positions(slot), r.result), r.rid


def test_many_slot_state_copies(gpu):
    from opencafemol_gb300 import synth
    specs = [synth.go_protein(n, 800 + n) for n in (40, 130, 77)]
    b = gpu.Batch(max_systems=4, max_total_beads=512, max_beads_per_system=200)
    slots = [b.admit(synth.build_system(s), s.pos, n_steps=10) for s in specs]
    xyz = np.concatenate([s.pos + 1.5 for s in specs])
    b.set_positions_many(slots, xyz)
    got = b.get_positions_many(slots)
    assert np.array_equal(got, xyz)
    assert np.array_equal(b.positions(slots[1]), specs[1].pos + 1.5)
    # reversed order round-trips too
    rev = slots[::-1]
    assert np.array_equal(b.get_positions_many(rev), np.concatenate([s.pos + 1.5 for s in specs[::-1]]))


def test_admission_by_device_memory_budget(gpu):
    """With a device-memory budget of about three systems' footprints the
    server never holds more than the budget, defers admissions until
    retirements free memory, and every request still completes with the
    result it has alone."""
    from opencafemol_gb300 import serving
    reqs = _requests(10, seed=5)
    fps = [r.system.footprint() for r in reqs]
    budget = int(sum(sorted(fps)[-3:]))
    server = serving.Server(max_systems=16, max_total_beads=16 * 700, max_beads_per_system=700,
                            chunk_steps=40, keep_results=True, hbm_budget_bytes=budget)
    st = server.serve(reqs, realtime=False)
    assert len(st.latencies_s) == 10 and st.failed == 0
    assert 0 < st.peak_resident_bytes <= budget
    assert st.waits_for_memory > 0
    r = reqs[7]
    alone = gpu.Batch(max_systems=1, max_total_beads=800, max_beads_per_system=700)
    slot = alone.admit(r.system, r.positions, temperature=r.temperature, seed=r.seed, n_steps=r.n_steps)
    alone.run(r.n_steps)
    assert np.array_equal(alone.positions(slot), r.result)
    tiny = serving.Server(max_systems=4, max_total_beads=4000, max_beads_per_system=700,
                          hbm_budget_bytes=min(fps) // 2)
    with pytest.raises(gpu.OCMError):
        tiny.serve(_requests(2, seed=6), realtime=False)


def test_blown_up_request_fails_alone(gpu):
    """A request whose system blows up completes as failed; the others in
    the same stream complete normally."""
    from opencafemol_gb300 import serving
    reqs = _requests(5, seed=8)
    x = reqs[2].positions.copy()
    x[-1] = x[0] + np.array([0.01, 0.0, 0.0])
    reqs[2].positions = x
    server = serving.Server(max_systems=8, max_total_beads=4000, max_beads_per_system=700, chunk_steps=30)
    st = server.serve(reqs, realtime=False)
    assert st.failed == 1 and len(st.latencies_s) == 5
    assert [r.failed for r in reqs] == [False, False, True, False, False]
