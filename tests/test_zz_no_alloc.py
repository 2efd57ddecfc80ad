"""ocm_batch_get_positions_many_noalloc against ocm_batch_get_positions_many,
both through the C ABI: the same positions on two calls in a row (with a
launch between them), in any slot order, and a clear error past its fixed
limits.  Named to run after every other test file, so it also passes with
the device state the other tests leave behind."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BEADS = 131072
MAX_SLOTS = 2048


def _batch(gpu, sizes, seed0):
    from opencafemol_gb300 import synth
    specs = [synth.go_protein(n, seed0 + k) for k, n in enumerate(sizes)]
    b = gpu.Batch(max_systems=len(specs) + 1, max_total_beads=sum(sizes) + 64, max_beads_per_system=800)
    slots = [b.admit(synth.build_system(s), s.pos, seed=11 + k, n_steps=10 ** 6) for k, s in enumerate(specs)]
    return b, slots


def _read(gpu, b, fn, slots, total):
    sl = np.ascontiguousarray(slots, np.int64)
    out = np.full((total, 3), np.nan)
    code = fn(b._h, len(sl), sl.ctypes.data_as(C.POINTER(C.c_int64)), out.ctypes.data_as(C.POINTER(C.c_double)))
    return code, out


def test_noalloc_matches_allocating_read_twice(gpu):
    lib = gpu.lib
    b, slots = _batch(gpu, [57, 400, 123, 800], seed0=3100)
    total = sum(b._n[s] for s in slots)
    b.run(25, sync=True)
    for _call in range(2):
        for order in (slots, slots[::-1], [slots[2], slots[2], slots[0]]):
            tot = sum(b._n[s] for s in order)
            ca, a = _read(gpu, b, lib.ocm_batch_get_positions_many, order, tot)
            cb, x = _read(gpu, b, lib.ocm_batch_get_positions_many_noalloc, order, tot)
            assert ca == 0 and cb == 0
            assert np.array_equal(a, x)
        b.run(25, sync=True)
    # and the Python wrapper agrees with the per-slot read
    got = b.get_positions_many_noalloc(slots)
    assert got.shape == (total, 3)
    assert np.array_equal(got[:57], b.positions(slots[0]))


def test_noalloc_limits(gpu):
    lib = gpu.lib
    b, slots = _batch(gpu, [800], seed0=3200)
    # 164 reads of an 800-bead slot exceed the bead limit
    reps = MAX_BEADS // 800 + 1
    code, _ = _read(gpu, b, lib.ocm_batch_get_positions_many_noalloc, [slots[0]] * reps, 800 * reps)
    assert code == 1
    assert f"at most {MAX_BEADS} beads" in lib.ocm_last_error().decode()
    b2, s2 = _batch(gpu, [40], seed0=3300)
    code, _ = _read(gpu, b2, lib.ocm_batch_get_positions_many_noalloc, [s2[0]] * (MAX_SLOTS + 1),
                    40 * (MAX_SLOTS + 1))
    assert code == 1
    assert f"at most {MAX_SLOTS} slots" in lib.ocm_last_error().decode()
    # the limits are exact: the largest allowed request succeeds
    n_ok = MAX_BEADS // 800
    code, x = _read(gpu, b, lib.ocm_batch_get_positions_many_noalloc, [slots[0]] * n_ok, 800 * n_ok)
    assert code == 0
    assert np.array_equal(x[:800], b.positions(slots[0])) and np.array_equal(x[-800:], x[:800])
