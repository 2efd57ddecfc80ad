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
    # the limits are exact: 2048 reads of a 64-bead slot are exactly 131072
    # beads in exactly 2048 slots and succeed; one more bead in the same
    # number of slots (2047 reads of 64 + one of 65) is refused
    b3, s3 = _batch(gpu, [64, 65], seed0=3400)
    code, x = _read(gpu, b3, lib.ocm_batch_get_positions_many_noalloc, [s3[0]] * MAX_SLOTS, 64 * MAX_SLOTS)
    assert 64 * MAX_SLOTS == MAX_BEADS
    assert code == 0
    assert np.array_equal(x[:64], b3.positions(s3[0])) and np.array_equal(x[-64:], x[:64])
    over = [s3[0]] * (MAX_SLOTS - 1) + [s3[1]]
    code, _ = _read(gpu, b3, lib.ocm_batch_get_positions_many_noalloc, over, MAX_BEADS + 1)
    assert code == 1
    assert f"at most {MAX_BEADS} beads" in lib.ocm_last_error().decode()
