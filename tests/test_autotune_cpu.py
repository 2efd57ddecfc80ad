"""Batch.autotune's selection logic with a stand-in batch (no GPU): every
candidate runs an untimed and a timed launch per round, the rounds
interleave the candidates, and the shape with the smallest mean is left
set."""
from opencafemol_gb300.engine import Batch


class _Shapes:
    """Launch times from a table by shape, minus a drift per launch."""

    def __init__(self, table, drift=0.0):
        self.table, self.drift = table, drift
        self.shape = [512, -1, 0]
        self.launches = []
        self.ms = 0.0

    def set_threads(self, t):
        self.shape[0] = t

    def set_list_smem(self, k):
        self.shape[1] = k

    def set_split(self, s):
        self.shape[2] = s

    def run(self, steps, sync=False):
        self.launches.append((tuple(self.shape), steps))
        self.ms = self.table[tuple(self.shape)] - self.drift * len(self.launches)

    def last_run_ms(self):
        return self.ms


def test_autotune_keeps_the_fastest_shape():
    table = {(512, 96, 512): 2.5, (1024, 96, 512): 3.0, (512, -1, 0): 2.7}
    fake = _Shapes(table)
    cands = ((512, 96, 512), (1024, 96, 512), (512, -1))
    res = Batch.autotune(fake, steps_per_trial=40, candidates=cands, rounds=2)
    assert (res["threads"], res["list_smem_kib"], res["split_beads"]) == (512, 96, 512)
    assert fake.shape == [512, 96, 512]
    # two launches per candidate and round, all of the requested length
    assert len(fake.launches) == 2 * 2 * 3 and all(s == 40 for _, s in fake.launches)
    # a two-entry candidate runs with split 0
    assert any(shape == (512, -1, 0) for shape, _ in fake.launches)
    assert [t["ms"] for t in res["trials"]] == [2.5, 3.0, 2.7]


def test_interleaved_rounds_spread_a_decaying_transient():
    # the faster shape comes first and its first timed launch falls in the
    # systems' early, slow transient: one round picks the slower shape,
    # three interleaved rounds pick the faster one
    class _Transient(_Shapes):
        def run(self, steps, sync=False):
            self.launches.append((tuple(self.shape), steps))
            self.ms = self.table[tuple(self.shape)] + 0.6 ** len(self.launches)

    table = {(512, 96, 512): 2.9, (1024, 96, 512): 3.0}
    cands = ((512, 96, 512), (1024, 96, 512))
    one = Batch.autotune(_Transient(table), steps_per_trial=10, candidates=cands, rounds=1)
    three = Batch.autotune(_Transient(table), steps_per_trial=10, candidates=cands, rounds=3)
    assert one["threads"] == 1024
    assert three["threads"] == 512
