"""Benchmark: bead-steps/s of the batched ensemble vs the plain path.

Workload (one GPU): 512 independent Go-model proteins, bead counts
log-uniform in [50, 800] (seeded), temperatures U[280, 360] K, dt = 10 fs,
gamma = 0.1 /ps, FP32 pair arithmetic with 64-bit fixed-point forces.  One
bench "step" is one persistent launch that advances every replica by
`--md-steps` MD steps.  Inputs are seeded synthetic systems (no dataset).

Printed JSON keys: value (device-timed,
state resident in HBM), e2e (through the public API with host buffers and
H2D/D2H copies inside the timed region), roofline of the dominant kernel,
cpu_baseline (the FP32 Verlet-list CPU restatement, OpenMP, on the whole
ensemble for a bounded number of steps), clocks sampled
during the timed region, and the plain single-system path on the same mix.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bead-steps/s batched vs plain on GB300 at <=1e-4 rel force err; p50/p99 latency"
N_SYSTEMS = 512
SIZE_LO, SIZE_HI = 50, 800
SEED = 2024


def local_device() -> int:
    return int(os.environ.get("LOCAL_RANK", "0"))


def _go_specs(params):
    from opencafemol_gb300 import synth
    return [synth.go_protein(int(n), int(sd), temperature=float(t)) for n, sd, t in params]


def go_specs(params, workers=None):
    """Seeded Go proteins for (beads, seed, temperature) triples, built in a
    process pool (spawn: the workers run numpy only and never load the
    engine library); the result is in the order of ``params``.  As with any
    spawn pool, a script that calls this must keep its own work under
    ``if __name__ == "__main__"`` (the workers import the main module)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    workers = workers or min(16, os.cpu_count() or 1)
    if len(params) < 32 or workers <= 1:
        return _go_specs(params)
    step = -(-len(params) // workers)
    chunks = [params[i:i + step] for i in range(0, len(params), step)]
    with cf.ProcessPoolExecutor(len(chunks), mp_context=mp.get_context("spawn")) as ex:
        return [s for part in ex.map(_go_specs, chunks) for s in part]


def ensemble_specs(count=N_SYSTEMS, seed=SEED):
    from opencafemol_gb300 import synth
    sizes = synth.ensemble_sizes(count, SIZE_LO, SIZE_HI, seed)
    temps = synth.ensemble_temperatures(count, seed)
    return go_specs([(int(n), seed * 1000 + k, float(t)) for k, (n, t) in enumerate(zip(sizes, temps))])


def clocks_rejected(summary: dict) -> bool:
    """A timed region whose clock record makes its number invalid: a
    hardware or thermal slowdown, or a median SM clock under 90% of the
    maximum with no reason active (sw_power_cap alone is kept)."""
    bad = {"hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"}
    reasons = set(summary.get("reasons", []))
    if reasons & bad:
        return True
    sm, smax = summary.get("sm_mhz"), summary.get("sm_max_mhz")
    return bool(sm and smax and sm < 0.9 * smax and not reasons)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.5)  # let the sampler start before the timed region
        except (FileNotFoundError, OSError):
            self.proc = None
        self.first = len(self.lines)
        self.last = None
        return self

    def stop_marker(self):
        """End of the timed region: later samples are not summarised."""
        self.last = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines[self.first:self.last]:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2():
    import torch
    buf = getattr(flush_l2, "buf", None)
    if buf is None:
        buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        flush_l2.buf = buf
    buf.fill_(1.0)
    torch.cuda.synchronize()


def pair_counts(specs):
    """Pairs within the largest cutoff at the initial positions (per system)."""
    out = []
    for s in specs:
        rc = 2.0
        d2 = np.sum((s.pos[:, None, :] - s.pos[None, :, :]) ** 2, axis=2)
        out.append(int(np.count_nonzero(np.triu(d2 < rc * rc, 1))))
    return np.array(out)


# Algorithmic FP32 work per pair within cutoff (EXV + DH, FMA = 2 flops),
# per bonded term and per bead update; counted from the kernel source.
FLOPS_PER_PAIR = 62
FLOPS_PER_BOND = 30
FLOPS_PER_ANGLE = 110
FLOPS_PER_DIHEDRAL = 160
FLOPS_PER_BEAD = 40
# integrator: read F (24), x (12), v (12), 1/m (4); write x (12), v (12),
# zero F (24)
BYTES_INTEGRATE_PER_BEAD = 100
# dram__bytes_read.sum + dram__bytes_write.sum of one timed k_batch launch of
# the default workload (100 MD steps of the 512-replica mix), from a
# `ncu --set full --clock-control none` capture of this script
K_BATCH_DRAM_BYTES = 21907712 + 512


def measured_hbm_gbs():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured (STREAM-style copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def batched_roofline(specs, K, launch_s, sm_max_mhz, traffic, sms=None):
    """Roofline object of one k_batch launch advancing every replica K steps.

    HBM view: compulsory bytes per MD step of a design that streams the
    state every step (positions + packed params in, 4 B per pair within the
    cutoff, 64-bit force write, bonded index/param records, integrator
    read/write of x, v, F, 1/m).  The persistent kernel keeps each system in
    shared memory, so its DRAM traffic ("traffic") is far below this.
    """
    beads = int(sum(s.n for s in specs))
    pc = pair_counts(specs)
    n_bond = sum(len(s.bonds) for s in specs)
    n_go = sum(len(s.contacts) for s in specs)
    n_ang = sum(len(s.fla_idx) for s in specs)
    n_dih = sum(len(s.fld_idx) for s in specs)
    pairs = int(pc.sum())
    bytes_step = int(beads * (16 + 24 + BYTES_INTEGRATE_PER_BEAD) + 4 * pairs
                     + 16 * n_go + 16 * n_bond + 16 * n_ang + 20 * n_dih)
    flops_step = int(pairs * FLOPS_PER_PAIR + (n_bond + n_go) * FLOPS_PER_BOND
                     + n_ang * FLOPS_PER_ANGLE + n_dih * FLOPS_PER_DIHEDRAL + beads * FLOPS_PER_BEAD)
    hbm_peak, hbm_src = measured_hbm_gbs()
    achieved_gbs = bytes_step * K / launch_s / 1e9
    achieved_tf = flops_step * K / launch_s / 1e12
    fp32_peak, sms = fp32_peak_tflops(sm_max_mhz, sms)
    return {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved_gbs / hbm_peak, "traffic": traffic, "peak_source": hbm_src,
            "kernel": "k_batch (persistent, shared-memory resident)",
            "algorithmic_bytes_per_launch": bytes_step * K,
            "bytes_per_bead_step": bytes_step / beads,
            "pairs_within_cutoff_per_bead": pairs / beads,
            "fp32": {"achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tf / fp32_peak, "flops_per_launch": flops_step * K,
                     "peak_source": f"{sms} SMs (read from the device) x 128 FP32 lanes x 2 flop x "
                                    f"max SM clock"}}


def rank_share(rank, world):
    """This rank's systems: one seeded ensemble of N_SYSTEMS x world Go
    proteins (the first N_SYSTEMS are the one-GPU workload), partitioned into
    whole systems by opencafemol_gb300.partition (largest first onto the
    least-loaded rank), about N_SYSTEMS per rank."""
    from opencafemol_gb300 import partition
    specs = ensemble_specs(count=N_SYSTEMS * world)
    if world == 1:
        return specs, specs
    sh = partition.shard([s.n for s in specs], rank, world)
    return [specs[k] for k in sorted(sh.indices)], specs


def run_ours(args, rank, world):
    import opencafemol_gb300 as ocm
    from opencafemol_gb300 import synth

    specs, all_specs = rank_share(rank, world)
    systems = [synth.build_system(s) for s in specs]
    beads = int(sum(s.n for s in specs))
    K = args.md_steps
    total_steps = (args.warmup + args.steps + 2) * K

    batch = ocm.Batch(max_systems=len(specs), max_total_beads=beads + 1024,
                      max_beads_per_system=SIZE_HI, device=local_device())
    total_beads = int(sum(s.n for s in all_specs))
    slots = [batch.admit(sysobj, s.pos, temperature=s.temperature, friction=s.friction,
                         step_size=s.dt, seed=1000 + k, n_steps=10 ** 12)
             for k, (sysobj, s) in enumerate(zip(systems, specs))]
    # warm-up launches first, so that the systems have relaxed from their
    # native structures before the autotuner times launch shapes; its trial
    # launches are real steps of the same systems; --threads fixes the shape
    tuned = None
    if args.threads:
        batch.set_threads(args.threads)
        batch.set_list_smem(args.list_smem)
        batch.set_split(args.split)
    for _ in range(args.warmup):
        batch.run(K, sync=True)
    if not args.threads:
        tuned = batch.autotune(steps_per_trial=K)
        batch.run(K, sync=True)

    import torch

    def timed_region():
        torch.cuda.synchronize()
        dist_barrier(world)
        times = []
        with ClockSampler(local_device()) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                flush_l2()
                batch.run(K, sync=True)
                times.append(batch.last_run_ms() / 1e3)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            clk.stop_marker()
        dist_barrier(world)
        return times, wall, clk

    times, wall, clk = timed_region()
    # a region that saw a hardware or thermal slowdown, or SM clocks well
    # below their maximum with no reason given (a clock lock left by someone
    # else), is measured once more; every rank takes the same decision
    remeasured = False
    if dist_max(float(clocks_rejected(clk.summary())), world) > 0:
        times, wall, clk = timed_region()
        remeasured = True
    value, dev_time = aggregate(beads, K, args.steps, float(np.sum(times)), world)
    ms_per_step = dev_time / args.steps * 1e3

    # ---- end to end through the public API with host buffers ----
    shape = ((tuned["threads"], tuned["list_smem_kib"], tuned["split_beads"]) if tuned
             else (args.threads, args.list_smem, args.split))
    e2e = run_e2e(batch, slots, beads, args, world)

    # ---- plain single-system path on a sample of the same mix ----
    plain = run_plain(ocm, specs, systems, args) if args.plain_sample > 0 else None
    plain_cfgs = (run_plain_configs(ocm, args)
                  if (args.cfg0_steps > 0 or args.cfg1_steps > 0 or args.cfg2_steps > 0) else None)

    # ---- served stream (continuous batching), p50/p99 completion latency ----
    serve = run_serving(ocm, args) if args.serve_requests > 0 and rank == 0 else None

    roof = batched_roofline(specs, K, dev_time / args.steps, clk.summary().get("sm_max_mhz"),
                            args.traffic_bytes if args.traffic_bytes > 0 else None)

    cpu = run_cpu_baseline(specs, md_steps=args.cpu_steps) if rank == 0 else None
    if cpu:
        cpu.pop("seconds", None)

    line = {
        "metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Go-model proteins)",
        "config": {"workload": f"batched ensemble: {len(all_specs)} Go proteins, N log-uniform "
                               f"[{SIZE_LO},{SIZE_HI}], T~U[280,360] K, dt=10 fs",
                   "replicas": len(all_specs), "beads": total_beads, "md_steps_per_launch": K,
                   "parallelism": (f"whole systems partitioned over {world} GPUs ({len(specs)} on rank 0, "
                                   f"largest first onto the least-loaded rank; no collective)"
                                   if world > 1 else "one GPU"),
                   "launch_shape": {"threads_per_cta": batch.threads(), "autotuned": tuned is not None,
                                    "list_smem_kib": shape[1], "split_beads": shape[2],
                                    "trials_ms": [t["ms"] for t in tuned["trials"]] if tuned else None},
                   "l2": "flushed (256 MiB write) between timed launches"},
        "e2e": e2e, "gpu_launches": args.steps, "roofline": roof, "cpu_baseline": cpu,
        "plain_path": plain,
        "plain_single_system": plain_cfgs,
        "serving": serve,
        "batched_vs_plain": value / world / plain["value"] if plain and plain.get("value") else None,
        "clocks": dict(clk.summary(), remeasured=remeasured), "wall_s": wall,
    }
    return line


def run_e2e(batch, slots, beads, args, world):
    """End to end through the public API with host buffers, as a host-driven
    loop runs it, on the batch of the device-timed leg (its trajectories
    continue): every step uploads every replica's positions from pinned host
    memory (one copy; the positions read back by the step before;
    velocities stay on the device), runs K MD steps and reads every
    replica's positions back (one copy)."""
    import torch
    K = args.md_steps
    host = torch.zeros((beads, 3), dtype=torch.float64).pin_memory()
    buf = host.numpy()
    batch.get_positions_many(slots, buf)
    for _ in range(2):
        batch.set_positions_many(slots, buf)
        batch.run(K, sync=True)
        batch.get_positions_many(slots, buf)
    torch.cuda.synchronize()
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.set_positions_many(slots, buf)
        batch.run(K, sync=True)
        batch.get_positions_many(slots, buf)
    t = dist_max(time.perf_counter() - t0, world)
    return {"value": dist_sum(float(beads), world) * K * args.steps / t, "unit": "bead-steps/s",
            "h2d_bytes_per_step": int(buf.nbytes), "d2h_bytes_per_step": int(buf.nbytes),
            "what": "positions H2D (pinned; the previous step's read-back) -> K MD steps -> positions D2H, "
                    "per step, continuing the device-timed batch"}


def run_serving(ocm, args):
    """Continuous batching on a bounded version of the serving stream: Go
    proteins of 30..2000 beads (log-uniform), T~U[280,360], Poisson arrivals
    at 200 req/s, admitted against a device-memory budget; step counts
    log-uniform in [1e4, 1e6] / scale and --serve-requests requests (the
    full stream is 10,000 requests at scale 1: about 1e12 bead-steps, some
    minutes of device time, too long for a benchmark run)."""
    from opencafemol_gb300 import serving, synth
    rng = np.random.default_rng(4242)
    n = args.serve_requests
    sizes = serving.log_uniform_int(rng, 30, 2001, n)
    steps = np.maximum(100, serving.log_uniform_int(rng, 1e4, 1e6, n) // args.serve_step_scale)
    temps = rng.uniform(280.0, 360.0, n)
    arrivals = serving.poisson_arrivals(n, args.serve_rate, seed=4243)
    reqs = []
    specs = go_specs([(int(sizes[k]), 90000 + k, float(temps[k])) for k in range(n)])
    for k, spec in enumerate(specs):
        reqs.append(serving.Request(rid=k, arrival=float(arrivals[k]), system=synth.build_system(spec),
                                    positions=spec.pos, temperature=float(temps[k]),
                                    n_steps=int(steps[k]), seed=k))
    server = serving.Server(max_systems=512, max_total_beads=300_000, max_beads_per_system=2048,
                            chunk_steps=args.serve_chunk, device=local_device(),
                            hbm_budget_bytes=int(args.serve_hbm_gib * 2 ** 30))
    st = server.serve(reqs, realtime=True).summary()
    offered = float(np.sum(sizes * steps) / arrivals[-1]) if n > 1 else None
    st.update({"offered_bead_steps_per_s": offered, "rate_req_per_s": args.serve_rate,
               "step_scale": args.serve_step_scale, "chunk_steps": args.serve_chunk,
               "launches": "balanced (the largest resident system does chunk_steps per launch)",
               "sizes": "log-uniform [30, 2000]", "steps": f"log-uniform [1e4, 1e6] / {args.serve_step_scale}",
               "requests_of_the_full_stream": 10000})
    return st


def run_plain(ocm, specs, systems, args):
    """Plain path: each system in its own Context, stepped one after another
    (CUDA-graph chunks), on an evenly spaced sample of the mix."""
    K = args.md_steps
    idx = np.linspace(0, len(specs) - 1, args.plain_sample).round().astype(int)
    bead_steps = 0
    t = 0.0
    for k in idx:
        s = specs[k]
        ctx = ocm.Context(systems[k], ocm.LangevinIntegrator(s.temperature, s.friction, s.dt, 31 + k),
                          device=local_device())
        ctx.setPositions(s.pos)
        ctx.setVelocitiesToTemperature(s.temperature, 5)
        ctx.step(K)  # warm: graph capture
        t0 = time.perf_counter()
        ctx.step(K * args.plain_chunks)
        t += time.perf_counter() - t0
        bead_steps += s.n * K * args.plain_chunks
    return {"value": bead_steps / t, "unit": "bead-steps/s", "systems_sampled": int(len(idx)),
            "what": "one Context per system, systems stepped sequentially (default engine: systems of "
                    "at most 512 beads on the one-system batched kernel, larger ones on the tiles)"}


def run_plain_configs(ocm, args):
    """The plain single-system path on the single-system shapes: a 60-bead
    Go protein (10 fs steps, non-periodic), a 20,000-bead HPS condensate
    slab (100 chains x 200 beads, 15 x 15 x 150 nm periodic box, HPS cutoff
    2.0 nm, Debye-Hueckel 3.5 nm on 20% charged beads) and the 200,000-bead
    slab of the same recipe (1000 chains, 30 x 30 x 300 nm).  The slabs
    start from a random packing, so they are relaxed first (untimed, strong
    friction, 2 fs steps).  Wall-clock timing around synchronous steps."""
    from opencafemol_gb300 import synth
    out = {}
    cases = []
    if args.cfg0_steps > 0:
        cases.append(("go_protein_60", synth.go_protein(60, 11), 0, args.cfg0_steps))
    if args.cfg1_steps > 0:
        cases.append(("hps_slab_20000", synth.hps_slab(100, 200, (15.0, 15.0, 150.0), slab_width=30.0, seed=7),
                      args.cfg1_relax, args.cfg1_steps))
    if args.cfg2_steps > 0:
        cases.append(("hps_slab_200000", synth.hps_slab(1000, 200, (30.0, 30.0, 300.0), slab_width=60.0, seed=7),
                      args.cfg1_relax, args.cfg2_steps))
    for name, spec, relax, steps in cases:
        system = synth.build_system(spec)
        pos = spec.pos
        if relax:
            # strong friction and 2 fs steps take the random packing's
            # overlaps out without heating the system
            rel = ocm.Context(system, ocm.LangevinIntegrator(spec.temperature, 5.0, 0.002, 3),
                              device=local_device())
            rel.setPositions(pos)
            rel.setVelocitiesToTemperature(spec.temperature, 3)
            rel.step(relax)
            pos = rel.getPositions()
            del rel
        ctx = ocm.Context(system, ocm.LangevinIntegrator(spec.temperature, spec.friction, spec.dt, 5),
                          device=local_device())
        ctx.setPositions(pos)
        ctx.setVelocitiesToTemperature(spec.temperature, 5)
        ctx.step(200)  # graph capture and the first list builds
        t0 = time.perf_counter()
        ctx.step(steps)
        t = time.perf_counter() - t0
        st = ctx.stats()
        out[name] = {"beads": int(spec.n), "steps": int(steps), "bead_steps_per_s": spec.n * steps / t,
                     "ns_per_day": steps / t * spec.dt * 86400 * 1e-3, "us_per_step": t / steps * 1e6,
                     "list_builds": int(st["list_builds"]), "tiles": int(st["tiles"]),
                     "charged_pairs": int(st["charged_pairs"]), "tile_cutoff_nm": round(st["tile_cutoff"], 4),
                     "engine": "one-system batched kernel" if st["one_system"] else "cluster-pair tiles",
                     "untimed_relaxation_steps": int(relax)}
    return out


def run_cpu_baseline(specs, md_steps=500, warm_steps=20, threads=0):
    """The CPU baseline: every replica of the workload advanced ``md_steps``
    steps by the FP32 Verlet-list restatement (oracle/cpu_baseline.cpp),
    OpenMP over replicas on all host cores.  Set-up and ``warm_steps``
    steps (the first list builds) are outside the timed region."""
    from oracle import oracle
    ens = oracle.CpuEnsemble(specs)
    cores = threads or oracle.CpuEnsemble.max_threads()
    ens.run(warm_steps, threads)
    t0 = time.perf_counter()
    ens.run(md_steps, threads)
    t = time.perf_counter() - t0
    beads = int(sum(s.n for s in specs))
    ens.close()
    return {"value": beads * md_steps / t, "unit": "bead-steps/s", "cores": int(cores), "kind": "port",
            "sample": f"all {len(specs)} replicas ({beads} beads) x {md_steps} MD steps; CPU restatement, "
                      f"not the reference: FP32 pair/bonded arithmetic, Verlet half list (0.3 nm skin, "
                      f"cell-grid build), OpenMP over replicas on {cores} threads", "seconds": t}


def fp32_peak_tflops(sm_max_mhz, sms=None):
    """FP32 FMA peak of the device: its SM count (read from the device
    unless given) x 128 FP32 lanes per SM (4 sub-partitions x 32 on this
    architecture) x 2 flops x the maximum SM clock sampled during the run."""
    if sms is None:
        import torch
        sms = torch.cuda.get_device_properties(local_device()).multi_processor_count
    mhz = sm_max_mhz or 2070.0
    return sms * 128 * 2 * mhz * 1e6 / 1e12, sms


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _dist_reduce(v, world, op_name):
    """A host value reduced over ranks (NCCL on the GPUs, gloo on the host)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def dist_max(v, world):
    return _dist_reduce(v, world, "MAX")


def dist_sum(v, world):
    return _dist_reduce(v, world, "SUM")


def aggregate(beads, md_steps, steps, dev_time_local, world):
    """Whole-job bead-steps/s: each rank advances its own share of the
    ensemble (``beads`` on this rank) by the same number of steps; the job's
    time is the slowest rank's."""
    t = dist_max(dev_time_local, world)
    return dist_sum(float(beads), world) * md_steps * steps / t, t


def run_reference(args, rank, world):
    """The reference arm: the reference's arithmetic lives in OpenMM, which
    is not installed on either machine, so the CPU restatement of the same
    force field stands in (oracle/cpu_baseline.cpp, all host threads).
    Each step advances the same workload as one step of this benchmark's own
    arm: every replica of the ensemble by ``--md-steps`` MD steps.  This
    process never loads the engine library."""
    if rank != 0:
        return None
    from oracle import oracle
    specs = ensemble_specs()
    beads = int(sum(s.n for s in specs))
    K = args.md_steps
    ens = oracle.CpuEnsemble(specs)
    cores = oracle.CpuEnsemble.max_threads()
    for _ in range(args.warmup):
        ens.run(K)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ens.run(K)
        times.append(time.perf_counter() - t0)
    ens.close()
    engine_loaded = "libocm_gb300" in Path("/proc/self/maps").read_text()
    total = float(np.sum(times))
    value = beads * K * args.steps / total
    cpu = {"value": value, "unit": "bead-steps/s", "cores": int(cores), "kind": "port",
           "sample": f"the whole workload: all {len(specs)} replicas ({beads} beads) x {K} MD steps per "
                     f"step; CPU restatement, not the reference (FP32, Verlet half list, OpenMP over "
                     f"replicas on {cores} threads)"}
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "bead-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Go-model proteins)",
            "config": {"workload": f"batched ensemble: {len(specs)} Go proteins, N log-uniform "
                                   f"[{SIZE_LO},{SIZE_HI}], T~U[280,360] K, dt=10 fs",
                       "replicas": len(specs), "beads": beads, "md_steps_per_step": K,
                       "note": "OpenMM (the reference's arithmetic) is not installed on either machine "
                               "(probed); the FP32 CPU restatement of the reference's force field "
                               "stands in"},
            "engine_library_loaded": engine_loaded,
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--md-steps", type=int, default=100)
    ap.add_argument("--plain-sample", type=int, default=24)
    ap.add_argument("--plain-chunks", type=int, default=2)
    ap.add_argument("--cpu-steps", type=int, default=500)  # MD steps of the whole ensemble, ~2 s
    ap.add_argument("--threads", type=int, default=0)   # fixes the launch shape (no autotuning) ...
    ap.add_argument("--list-smem", type=int, default=-1)  # ... with this list budget (KiB, -1 = no cap)
    ap.add_argument("--split", type=int, default=512)     # ... and this CTA split size (beads)
    ap.add_argument("--serve-requests", type=int, default=1000)
    ap.add_argument("--traffic-bytes", type=float, default=K_BATCH_DRAM_BYTES,
                    help="DRAM bytes per k_batch launch (ncu), reported as roofline.traffic")
    ap.add_argument("--cfg0-steps", type=int, default=10000)
    ap.add_argument("--cfg1-steps", type=int, default=2000)
    ap.add_argument("--cfg1-relax", type=int, default=3000)
    ap.add_argument("--cfg2-steps", type=int, default=1000)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-step-scale", type=int, default=20)
    ap.add_argument("--serve-hbm-gib", type=float, default=4.0)
    ap.add_argument("--serve-chunk", type=int, default=100)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line))
        return
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    line = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
