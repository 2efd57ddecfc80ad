"""Trajectories matched statistically against the FP64 oracle.

MD is chaotic, so the GPU's trajectories cannot follow the oracle's step for
step over long runs; what must agree is the ensemble they sample.  A Go
protein built with the 60-bead single-system recipe (harmonic bonds, Go
contacts, flexible-local angles and dihedrals, excluded volume,
Debye-Hueckel; 300 K, gamma = 0.1 /ps, dt = 10 fs) is run as independent
replicas by the batched engine, by the plain engine and, with other noise
seeds, by the oracle's FP64 Langevin integrator (the same leapfrog scheme, Philox noise).  From
Maxwell-Boltzmann velocities at the native structure, each replica is
equilibrated and then sampled every 50 steps.  Per-replica means of the
kinetic temperature, the radius of gyration and the fraction of native
contacts formed (r < 1.5 r0; the chain is mostly unfolded at
300 K) must agree between the two engines within
4.5 combined standard errors (replica means are independent), and their
sample spreads within 25 %."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOLTZ = 0.00831446261815324
REPLICAS = 16
EQUIL = 2000
SAMPLES = 200
EVERY = 50


def _observables(spec, x, v):
    m = spec.masses
    t_kin = float(np.sum(m[:, None] * v * v) / (3 * spec.n * BOLTZ))
    c = x - x.mean(axis=0)
    rg = float(np.sqrt(np.mean(np.sum(c * c, axis=1))))
    ij = np.asarray(spec.contacts, np.int64)
    r = np.linalg.norm(x[ij[:, 0]] - x[ij[:, 1]], axis=1)
    q = float(np.mean(r < 1.5 * np.asarray(spec.go_r0)))
    return t_kin, rg, q


def _mb_velocities(spec, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(spec.n, 3)) * np.sqrt(BOLTZ * spec.temperature / spec.masses)[:, None]
    return v.astype(np.float32).astype(np.float64)


def _gpu_samples(gpu, spec):
    from opencafemol_gb300 import synth
    system = synth.build_system(spec)
    batch = gpu.Batch(max_systems=REPLICAS, max_total_beads=REPLICAS * 64, max_beads_per_system=64)
    slots = [batch.admit(system, spec.pos, velocities=_mb_velocities(spec, 100 + k),
                         temperature=spec.temperature, friction=spec.friction, step_size=spec.dt,
                         seed=500 + k, n_steps=EQUIL + SAMPLES * EVERY)
             for k in range(REPLICAS)]
    batch.run(EQUIL, sync=True)
    out = np.zeros((REPLICAS, SAMPLES, 3))
    for s in range(SAMPLES):
        batch.run(EVERY, sync=True)
        for k, slot in enumerate(slots):
            out[k, s] = _observables(spec, batch.positions(slot), batch.velocities(slot))
    return out


def _plain_samples(gpu, spec):
    from opencafemol_gb300 import synth
    system = synth.build_system(spec)
    out = np.zeros((REPLICAS, SAMPLES, 3))
    for k in range(REPLICAS):
        ctx = gpu.Context(system, gpu.LangevinIntegrator(spec.temperature, spec.friction, spec.dt, 700 + k),
                          engine="tiles")
        ctx.setPositions(spec.pos)
        ctx.setVelocities(_mb_velocities(spec, 100 + k))
        ctx.step(EQUIL)
        for s in range(SAMPLES):
            ctx.step(EVERY)
            out[k, s] = _observables(spec, ctx.getPositions(), ctx.getVelocities())
    return out


def _oracle_samples(spec):
    from oracle import oracle

    def one(k):
        x = spec.pos.copy()
        v = _mb_velocities(spec, 100 + k)
        res = np.zeros((SAMPLES, 3))
        oracle.simulate(spec, x, v, EQUIL, seed=9000 + k)
        step = EQUIL
        for s in range(SAMPLES):
            oracle.simulate(spec, x, v, EVERY, seed=9000 + k, step0=step)
            step += EVERY
            res[s] = _observables(spec, x, v)
        return res

    with ThreadPoolExecutor(max_workers=REPLICAS) as ex:
        return np.stack(list(ex.map(one, range(REPLICAS))))


@pytest.mark.parametrize("engine", ["batched", "plain"])
def test_ensembles_match_oracle(gpu, engine):
    from opencafemol_gb300 import synth
    spec = synth.go_protein(60, 11)
    assert len(spec.contacts) >= 10
    g = _gpu_samples(gpu, spec) if engine == "batched" else _plain_samples(gpu, spec)
    c = _oracle_samples(spec)
    names = ("temperature", "radius of gyration", "native contact fraction")
    for k, name in enumerate(names):
        mg, mc = g[:, :, k].mean(axis=1), c[:, :, k].mean(axis=1)
        se = np.sqrt(mg.var(ddof=1) / len(mg) + mc.var(ddof=1) / len(mc))
        diff = abs(mg.mean() - mc.mean())
        assert diff <= 4.5 * se + 1e-9, (name, mg.mean(), mc.mean(), se)
        sg, sc = g[:, :, k].std(), c[:, :, k].std()
        assert abs(sg - sc) <= 0.25 * max(sg, sc), (name, sg, sc)
    # both thermostats hold the bath temperature
    for arr in (g, c):
        t = arr[:, :, 0].mean(axis=1)
        assert abs(t.mean() - spec.temperature) <= 4.5 * t.std(ddof=1) / np.sqrt(len(t)) + 0.02 * spec.temperature
