"""The timed CPU baseline (oracle/cpu_baseline.cpp) computes the same force
field as the FP64 oracle: it is a baseline, so FP32 tolerances apply, but a
wrong term or a missing pair would show here."""
import numpy as np
import pytest


def _rel(f, ref):
    fr = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fr ** 2))
    return float(np.max(np.linalg.norm(f - ref, axis=1) / np.maximum(fr, floor)))


@pytest.mark.parametrize("n,seed", [(60, 1), (400, 2), (800, 3)])
def test_go_protein_matches_oracle(n, seed):
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.go_protein(n, seed, temperature=320.0)
    ens = oracle.CpuEnsemble([spec])
    f, e = ens.evaluate(0)
    fr, er = oracle.evaluate(spec, fp32_cutoff=False)
    # plain FP32 arithmetic (r - r0 of stiff bonds cancels): 1e-3 per bead
    assert _rel(f, fr) < 1e-3
    ref = np.array(list(er.values())[:8])
    assert np.allclose(e, ref, rtol=2e-5, atol=1e-3)


def test_periodic_hps_matches_oracle():
    from opencafemol_gb300 import synth
    from oracle import oracle
    spec = synth.hps_slab(8, 40, (8.0, 8.0, 30.0), slab_width=8.0, seed=5)
    ens = oracle.CpuEnsemble([spec])
    f, e = ens.evaluate(0)
    fr, er = oracle.evaluate(spec, fp32_cutoff=False)
    ref = np.array(list(er.values())[:8])
    # an unrelaxed random packing: huge cancelling overlap forces, so the
    # comparison is on the RMS error and the energies
    assert np.sqrt(np.mean(np.sum((f - fr) ** 2, 1))) < 1e-4 * np.sqrt(np.mean(np.sum(fr ** 2, 1)))
    assert np.allclose(e, ref, rtol=1e-4, atol=1e-2)


def test_ensemble_runs_and_rebuilds_lists():
    from opencafemol_gb300 import synth
    from oracle import oracle
    specs = [synth.go_protein(n, 40 + n, temperature=300.0) for n in (50, 120, 300)]
    ens = oracle.CpuEnsemble(specs)
    x0 = [ens.positions(k) for k in range(3)]
    ens.run(300, threads=2)
    for k, s in enumerate(specs):
        x = ens.positions(k)
        assert np.all(np.isfinite(x))
        assert 0 < np.max(np.abs(x - x0[k])) < 5.0
        # bonds stay near 0.38 nm at 300 K
        d = np.linalg.norm(x[s.bonds[:, 0]] - x[s.bonds[:, 1]], axis=1)
        assert np.all(np.abs(d - 0.38) < 0.08)
