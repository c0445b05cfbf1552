"""Benchmark of the per-step particle path: particle-steps/s on one GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl tfg|reference]

Default workload "ensemble": 256 independent cell-sorting simulations (particle counts
log-uniform in [500, 50,000], A-B Morse depth uniform in [0.1, 2.0], box side for density
0.5, Gaussian random force 0.1) held in one device arena.  A "step" is one engine step of
every simulation of the batch (re-bin, fused pair pass, advance, FP64 per-simulation
totals), K steps replayed from captured CUDA graphs.  The arena (about 2.75M particles,
several hundred MB) is larger than L2, so L2 is not flushed.

value     = batched particle-steps/s (sum of N_i over the batch x K / CUDA-event time on
            the engine's stream, max over ranks).
plain_gpu = the same simulations run one at a time, each in its own engine (same kernels,
            same graphs), the "plain one-simulation-at-a-time GPU path".
e2e       = the whole job through the C ABI with host buffers: load every simulation from
            host arrays, run --e2e-steps steps, download positions and velocities.
serving   = a bounded sample of the served stream (Poisson arrivals at 200/s, 60/40 cell
            sorting / DPD droplets, 1,000-200,000 particles, 100-5,000 steps): achieved
            particle-steps/s, p50/p99 completion latency.
roofline  = the pair kernel against the measured FP32 FMA peak (tfg_probe_fp32_tflops), and
            the whole step against the measured HBM bandwidth.
cpu_baseline: the CPU restatement of the reference engine (threaded, all host cores) on a
            bounded sample of the same simulations.
Other workloads (--workload dpd_droplets | bonded_fluid | cell_sorting) time one
simulation with L2 flushed between steps; --workload served runs only the served stream.
--impl reference: the CPU restatement of the reference engine timed on the host cores (the
            reference itself cannot be built: its Magnum/Corrade/libsbml submodules are
            empty and it needs GL/GLFW/assimp).
For N>1 (torchrun) every rank runs an independent replica (no data-path exchange between
simulations): scaling "weak", value = all ranks' particle-steps / the slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tissue-forge_gb300"))

import numpy as np  # noqa: E402

WORKLOADS = {
    "ensemble": dict(desc="batched ensemble: 256 independent cell-sorting simulations, N log-uniform in "
                          "[500, 50000], A-B Morse depth U[0.1, 2.0], density 0.5, cutoff 3, random force 0.1, "
                          "overdamped dt 0.005", bytes_per_particle=48),
    "served": dict(desc="served stream: Poisson arrivals 200/s, 60/40 cell-sorting / DPD-droplet simulations, "
                        "N log-uniform in [1000, 200000], steps U[100, 5000]", bytes_per_particle=64),
    "dpd_droplets": dict(desc="DPD droplets with Fickian flux: 100,000 particles, box 40, cutoff 1, "
                              "alpha 10 gamma 4.5 sigma 3, Fick k 0.5, dt 0.01", bytes_per_particle=88),
    "dpd_droplets_species": dict(desc="the DPD droplets with three species, each diffusing by Fick (k 0.5, 0.2, "
                                      "0.1 with decay 0.05): 100,000 particles, box 40, cutoff 1",
                                 bytes_per_particle=104),
    "bonded_fluid": dict(desc="LJ 12-6 fluid in chains of 16 with harmonic bonds and angles: 2,000,000 particles "
                              "at density 0.85, cutoff 2.5, dt 0.002", bytes_per_particle=80),
    "cell_sorting": dict(desc="cell sorting: 4,000 particles, box 20, cutoff 3, shifted Morse, overdamped",
                         bytes_per_particle=48),
    "lj_fluid": dict(desc="LJ 12-6 fluid from a jittered lattice: 2,000,376 particles at density 0.85, cutoff 2.5, "
                          "T 0.5, dt 0.002, cell lists (cell edge >= cutoff)", bytes_per_particle=64),
    "lj_fluid_verlet": dict(desc="the lj_fluid workload in Verlet mode (engine_flag_verlet): cell edge >= 1.2 cutoff, "
                                 "re-binning only when 2 maxdx > skin, device pair lists between rebuilds",
                            bytes_per_particle=64),
}

# Algorithmic flops per interacting pair (one evaluation serving both particles) and per
# particle integrate, as counted for the roofline.
FLOPS = dict(table=50, dpd=45, flux=12, density=12, bond=45, angle=75, integrate_newtonian=18,
             integrate_overdamped=15)


def make_workload(name, seed, n=None, relax=None):
    """The named workload at its configured size, or scaled to n particles (same density)."""
    from tfg import configs
    if name == "dpd_droplets":
        if n:
            scale = (n / 100_000) ** (1.0 / 3.0)
            return configs.dpd_droplets(n=n, side=40.0 * scale, radius=12.0 * scale, seed=1 + seed)
        return configs.dpd_droplets(seed=1 + seed)
    if name == "dpd_droplets_species":
        return configs.dpd_droplets_species(seed=1 + seed)
    if name == "bonded_fluid":
        w = configs.bonded_fluid(n=n or 2_000_000, seed=2 + seed)
        if relax is not None:
            w.relax_steps = relax
        return w
    if name == "cell_sorting":
        if n:
            return configs.cell_sorting(n=n, side=20.0 * (n / 4000) ** (1.0 / 3.0), seed=seed)
        return configs.cell_sorting(seed=seed)
    if name == "lj_fluid":
        return configs.lj_fluid(n=n or 2_000_000, seed=5 + seed)
    if name == "lj_fluid_verlet":
        return configs.verlet(configs.lj_fluid(n=n or 2_000_000, seed=5 + seed), skin=VERLET_SKIN)
    raise SystemExit("unknown workload " + name)


VERLET_SKIN = 0.2   # cell edge >= (1 + VERLET_SKIN) * cutoff for the Verlet workload


def timed_rate(eng, n, steps, warmup, flush, stream, world=1):
    """particle-steps/s of `steps` single steps, L2 flushed before each (CUDA events)."""
    import torch
    for _ in range(warmup):
        eng.step(1, sync=False)
    eng.set_phase_timing(False)
    eng.step(2)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()
        ev[k][0].record(stream)
        eng.step(1, sync=False)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    return world * n * steps / (sum(a.elapsed_time(b) for a, b in ev) * 1e-3)


def pair_flops(w):
    f = FLOPS["density"] if not (w.flags & 2) else 0
    kinds = {spec.kind for spec in w.pots.values()}
    if "dpd" in kinds:
        f += FLOPS["dpd"]
    elif kinds:
        f += FLOPS["table"]
    if w.fluxes:
        f += FLOPS["flux"] * len(w.fluxes)
    return f


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason sampling during the timed region."""

    def __init__(self, index, path):
        self.path = path
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference_rate(w, threads, budget_s, max_steps=200):
    """Particle-steps/s of the CPU restatement on the host cores (bounded sample)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from tfg.engine import setup_model
    e = O.OracleEngine(w.desc(), 0, threads, signature=False)
    keep = setup_model(e, w)
    e.step(1)   # warm-up
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        e.step(1)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    del keep
    return w.n * steps / dt, steps, dt



def hbm_peak():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def clock_path(name):
    """Where the nvidia-smi clock samples go (TFG_CLOCKS_DIR, else the temporary directory)."""
    import tempfile
    return os.path.join(os.environ.get("TFG_CLOCKS_DIR") or tempfile.gettempdir(), name)


def fp32_peak(dev):
    import ctypes as C
    from tfg import lib
    peak = C.c_double(0.0)
    lib().tfg_probe_fp32_tflops(dev, C.byref(peak))
    return peak.value


# DRAM traffic of the tiled pair kernel per particle of the arena: one ncu capture of the
# 256-simulation ensemble pass (2,902,298 particles) read 141.3 MB and wrote 26.7 MB
# (dram__bytes_read.sum + dram__bytes_write.sum), 57.9 B per particle.  The traffic is the
# particle data read and the forces written, so it scales with the particles, not the pairs.
PAIR_TRAFFIC_BYTES_PER_PARTICLE = 57.9


def launches_per_step(has_bonds=False, has_angles=False):
    # tick, 7 binning kernels (count, 3 scan passes, place, rank, scatter), the tiled pair
    # kernel and its overflow kernel, bonds, angles, advance
    return 1 + 7 + 2 + int(has_bonds) + int(has_angles) + 1


def ensemble_sample(ws, count):
    """Every k-th simulation of the ensemble, `count` of them (the bounded CPU sample)."""
    k = max(1, len(ws) // count)
    return ws[::k][:count]


def cpu_rate_sims(ws, threads, budget_s, max_steps=50):
    """Particle-steps/s of the CPU restatement over simulations run one after another."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from tfg.engine import setup_model
    tot_ps, tot_t, steps_done = 0.0, 0.0, []
    per_sim = budget_s / max(1, len(ws))
    for w in ws:
        e = O.OracleEngine(w.desc(), 0, threads, signature=False)
        keep = setup_model(e, w)
        e.step(1)
        t0 = time.perf_counter()
        k = 0
        while k < max_steps:
            e.step(1)
            k += 1
            if time.perf_counter() - t0 > per_sim:
                break
        dt = time.perf_counter() - t0
        tot_ps += w.n * k
        tot_t += dt
        steps_done.append(k)
        del keep, e
    return tot_ps / tot_t, steps_done, tot_t


CPU_SAMPLE_SIMS = 16     # simulations of the ensemble in the bounded CPU sample
CPU_SAMPLE_ROUNDS = 12   # timed rounds; each round steps every sampled simulation once


def ensemble_cpu_sample(sims):
    """The bounded CPU sample of the ensemble, the same for the reference arm and the GPU
    line's cpu_baseline: every (sims/16)-th simulation of the ensemble in its natural order."""
    from tfg import configs
    return ensemble_sample(configs.ensemble(count=sims), CPU_SAMPLE_SIMS)


def cpu_rate_rounds(ws, threads, rounds, warmup):
    """Particle-steps/s of the CPU restatement (threaded, as the reference's runners) over
    `rounds` rounds in which every simulation of `ws` takes one engine step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from tfg.engine import setup_model
    engines = []
    for w in ws:
        e = O.OracleEngine(w.desc(), 0, threads, signature=False)
        engines.append((e, setup_model(e, w), w.n))
    for _ in range(warmup):
        for e, _, _ in engines:
            e.step(1)
    ps, t = 0.0, 0.0
    for _ in range(rounds):
        t0 = time.perf_counter()
        for e, _, n in engines:
            e.step(1)
            ps += n
        t += time.perf_counter() - t0
    return ps / t, t


def ensemble_config(sims, world, n_all):
    """`config` of the ensemble line: the workload only (sims per rank, the whole job's
    simulations and particles), the same in both arms."""
    return {"workload": "ensemble", "description": WORKLOADS["ensemble"]["desc"], "sims_per_rank": sims,
            "sims_all_ranks": sims * world, "n_particles_all_ranks": n_all,
            "l2": "working set larger than L2 (not flushed)", "parallelism": "replicas%d" % world}


def run_reference(args, rank, world):
    """The reference's CPU engine on the host cores: the CPU restatement (the reference
    itself cannot be built here), threaded like the reference's runners, on a bounded sample
    of the GPU line's workload, with the GPU line's config, metric and unit."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if args.workload in ("ensemble", "served"):
        from tfg import configs
        ws = ensemble_cpu_sample(args.sims)
        ns, _ = configs.ensemble_sizes(args.sims * world)
        config = ensemble_config(args.sims, world, int(np.sum(ns)))
        rounds = CPU_SAMPLE_ROUNDS
        sample = ("%d of the %d simulations (every %dth, %d particles), %d rounds of one engine step each, "
                  "threaded CPU restatement of the reference engine" % (
                      len(ws), args.sims, max(1, args.sims // CPU_SAMPLE_SIMS), sum(w.n for w in ws), rounds))
    else:
        ws = [make_workload(args.workload, 0, args.n or None, args.relax)]
        config = {"workload": args.workload, "description": WORKLOADS[args.workload]["desc"], "n_particles": ws[0].n}
        rounds = min(args.steps, 30)
        sample = "%d engine steps of the %s workload, threaded CPU restatement" % (rounds, args.workload)
    value, t = cpu_rate_rounds(ws, threads, rounds, args.warmup)
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": rounds, "warmup": args.warmup, "ms_per_step": 1e3 * t / rounds,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference", "config": config,
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batched_same_requests(reqs, dev, steps=30):
    """The served sample's requests run without the serving loop: all resident at once, one
    batch per model family (as the server's lanes, each on its own stream, both in flight
    together), every simulation stepped `steps` steps.  Its particle-steps/s is what the GPU
    gives this request mix when nothing arrives, finishes or is re-laid out; the served
    throughput is stated against it."""
    from tfg.engine import Batch, setup_model
    cache, groups = {}, {}
    for r in reqs:
        groups.setdefault((r.workload.max_type, r.workload.nr_species), []).append(r.workload)
    batches = []
    for (mt, ns), ws in groups.items():
        b = Batch(mt, ns, dev)
        for w in ws:
            s = b.add_sim(w.desc(device=dev))
            b._keep.extend(setup_model(s, w, pot_cache=cache))
        b.step(3)   # layout, autotune, graph capture
        batches.append(b)
    n = sum(r.workload.n for r in reqs)
    t0 = time.perf_counter()
    for b in batches:
        b.step(steps, sync=False)
    for b in batches:
        b.sync()
    dt = time.perf_counter() - t0
    for b in batches:
        b.close()
    return {"particle_steps_per_s": n * steps / dt, "particles": n, "steps": steps, "batches": len(batches),
            "how": "the same requests, all resident, one batch per model family, %d steps each, host clock "
                   "around both batches" % steps}


def serve_sample(args, dev, count, rate=200.0, policy="sjf", compare_batched=False):
    """A bounded sample of the served stream: the first `count` requests of the Poisson
    stream at `rate` requests/s, with their particles generated before the clock starts
    (client-side data); a stream of more than 1,000 requests generates each request's
    particles when it arrives instead, inside the clock."""
    from tfg import configs
    from tfg.serving import Request, Server, summarize
    reqs = []
    lazy = count > 1000   # a long stream builds each request when it arrives
    for r in configs.served_requests(count=count, rate=rate, seed=args.seed):
        if lazy:
            reqs.append(Request(len(reqs), r["t"], None, r["steps"], make=lambda r=r: configs.request_workload(r)))
        else:
            reqs.append(Request(len(reqs), r["t"], configs.request_workload(r), r["steps"]))
    t_first = reqs[0].t_arrival
    for r in reqs:
        r.t_arrival -= t_first
    srv = Server(budget_bytes=150 << 30, max_particles=args.serve_particles, quantum=args.quantum, device=dev,
                 keep_results=False, policy=policy)
    done = srv.run(reqs)
    s = summarize(done)
    st = srv.stats()
    s["host_s"] = {"admit": st["admit_s"], "launch": st["launch_s"], "retire": st["retire_s"],
                   "batch_busy": st["busy_s"], "batch_gap": st["gap_s"],
                   "note": "host time of the native server: recording requests into batches, starting "
                           "chunks (arena re-layout after membership changes), retiring; batch_busy and "
                           "batch_gap sum over the batches the time from a chunk's start to its observed "
                           "completion and from there to the batch's next chunk"}
    if compare_batched:
        s["batched_same_requests"] = batched_same_requests(reqs, dev)
        ref = s["batched_same_requests"]["particle_steps_per_s"]
        s["served_over_batched"] = s["achieved_particle_steps_per_s"] / ref
        if s["backlogged_particle_steps_per_s"]:
            s["backlogged_over_batched"] = s["backlogged_particle_steps_per_s"] / ref
    s.update({"policy": policy, "max_concurrent": srv.max_concurrent, "chunks": srv.chunks, "quantum": args.quantum,
              "max_particles_in_flight": args.serve_particles, "budget_bytes": 150 << 30,
              "rate_per_s": rate,
              "sample": "first %d of the 10,000 requests (arrivals re-based to t=0)" % count})
    return s


def run_ensemble(args, rank, world, dev, dist):
    import torch
    from tfg import configs
    from tfg.engine import Batch, Engine, setup_model
    from tfg.sharding import max_over_ranks, shard
    # an ensemble of sims x world simulations, LPT-partitioned over the ranks by work
    ns_all, _ = configs.ensemble_sizes(args.sims * world)
    ws = configs.ensemble(count=args.sims * world, indices=shard(ns_all, rank, world))
    n_tot = sum(w.n for w in ws)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    cache = {}

    def make_batch():
        b = Batch(2, 0, dev)
        b.set_stream(stream.cuda_stream)
        sims = []
        for w in ws:
            s = b.add_sim(w.desc(device=dev))
            b._keep.extend(setup_model(s, w, pot_cache=cache))
            sims.append(s)
        return b, sims

    b, sims = make_batch()
    split = tune(b, args)
    tuning = b.tuning()
    b.step(args.warmup)
    cnt0, _ = b.pair_signature()
    pairs0 = int(cnt0.sum()) // 2
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b.set_phase_timing(False)   # the timed steps carry no phase stamps
    b.step(2)                   # re-capture the step graphs without them
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev, clock_path("clocks_bench.csv")) as clk:
        e0.record(stream)
        b.step(args.steps, sync=False)
        e1.record(stream)
        torch.cuda.synchronize()
    b.sync()
    if dist is not None:
        dist.barrier()
    t_ms = max_over_ranks(e0.elapsed_time(e1), dist, device="cuda")
    n_all = int(np.sum(ns_all))
    value = n_all * args.steps / (t_ms * 1e-3)
    step_ms = t_ms / args.steps
    # phase split and pair-kernel time from a few stamped steps after the timed region
    b.set_phase_timing(True)
    b.step(2)
    phase = np.zeros(4)
    for _ in range(5):
        b.step(1)
        phase += np.array(b.phase_ms())
    phase /= 5
    cnt1, _ = b.pair_signature()
    pairs = 0.5 * (pairs0 + int(cnt1.sum()) // 2)
    b.close()

    # plain path: every simulation alone in its own engine, one after another
    kp = args.plain_steps
    plain_ps, plain_ms = 0.0, 0.0
    for w in ws:
        e = Engine(w.desc(device=dev))
        keep = setup_model(e, w, pot_cache=cache)
        e.set_stream(stream.cuda_stream)
        tune(e, args)
        e.step(3)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        e.step(kp, sync=False)
        a1.record(stream)
        torch.cuda.synchronize()
        e.sync()
        plain_ms += a0.elapsed_time(a1)
        plain_ps += w.n * kp
        e.close()
        del keep
    plain_ms = max_over_ranks(plain_ms, dist, device="cuda")
    plain = {"value": n_all * kp / (plain_ms * 1e-3), "unit": "particle-steps/s",
             "ms_per_round": plain_ms / kp, "steps_per_sim": kp,
             "how": "each simulation alone in its own engine (same kernels, CUDA graphs), one after another"}

    # end to end: the whole job through the C ABI with host arrays
    E = args.e2e_steps or ws[0].steps
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    host = [(pin(w.x), pin(w.type), pin(w.radius), pin(w.imass)) for w in ws]
    outs = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b2 = Batch(2, 0, dev)
    b2.set_stream(stream.cuda_stream)
    sims2 = []
    for w, (hx, ht, hr, hi) in zip(ws, host):
        s = b2.add_sim(w.desc(device=dev))
        keep = setup_model(s, w, pot_cache=cache)
        b2._keep.extend(keep)
        s.load(hx, type=ht, radius=hr, imass=hi)
        sims2.append(s)
    b2.step(E)
    for s in sims2:
        outs.append(s.download())
    t_e2e = time.perf_counter() - t0
    b2.close()
    bi = n_tot * (12 + 4 + 4 + 4)
    bo = n_tot * (12 + 12 + 12 + 12 + 4 + 4)
    t_e2e = max_over_ranks(t_e2e, dist, device="cuda")
    e2e = {"value": n_all * E / t_e2e, "unit": "particle-steps/s",
           "h2d_bytes_per_step": bi / E, "d2h_bytes_per_step": bo / E, "steps": E,
           "how": "Batch + tfg_batch_add_sim/load_particles for all %d simulations from host arrays, "
                  "tfg_step(%d), tfg_batch_download of each (x, xrel, v, f, cell, density); model set-up "
                  "(potential tables cached from the batched run) inside the timed region" % (len(ws), E)}

    # roofline: the pair kernel against the FP32 peak, the step against HBM
    fl_pair = pairs * (FLOPS["table"] + FLOPS["density"])
    achieved = fl_pair / (phase[1] * 1e-3) / 1e12
    peak = fp32_peak(dev)
    hbm, hbm_src = hbm_peak()
    bytes_alg = n_tot * WORKLOADS["ensemble"]["bytes_per_particle"]
    roof = {"bound": "fp32", "kernel": pair_kernel_name(split), "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
            "peak_source": "measured live (tfg_probe_fp32_tflops, FFMA chains)",
            "flops_per_launch": fl_pair, "pairs_per_step": pairs,
            "flops_per_pair": FLOPS["table"] + FLOPS["density"], "kernel_ms": phase[1],
            "traffic": PAIR_TRAFFIC_BYTES_PER_PARTICLE * n_tot,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of the tiled "
                              "kernel on this ensemble (57.9 B per particle), scaled by the particles",
            "algorithmic_bytes_per_launch": n_tot * 56,
            "step_hbm": {"achieved_gbs": bytes_alg / (step_ms * 1e-3) / 1e9, "peak_gbs": hbm,
                         "peak_source": hbm_src, "frac": bytes_alg / (step_ms * 1e-3) / 1e9 / hbm,
                         "bytes_per_step": bytes_alg}}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the same sample and timing as bench.py --impl reference
        threads = os.cpu_count() or 1
        sample = ensemble_cpu_sample(args.sims)
        rate, dt = cpu_rate_rounds(sample, threads, CPU_SAMPLE_ROUNDS, args.warmup)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": "%d of the %d simulations (every %dth, %d particles), %d rounds of one engine step each, "
                         "threaded CPU restatement of the reference engine, %.1f s" % (
                             len(sample), args.sims, max(1, args.sims // CPU_SAMPLE_SIMS), sum(w.n for w in sample),
                             CPU_SAMPLE_ROUNDS, dt)}
    workloads = None
    if rank == 0 and args.sub_workloads:
        workloads = {name: measure_workload(name, dev, stream, args.sub_steps, args.warmup, args)
                     for name in args.sub_workloads.split(",")}
    serving = serve_sample(args, dev, args.requests, compare_batched=True) if (rank == 0 and args.requests > 0) else None
    if serving is not None and args.sustained_requests > 0:
        # the same stream at an arrival rate the GPU sustains (about half its served capacity),
        # so the latencies show service time rather than backlog
        work = serving["particle_steps"] / serving["requests"]
        rate = 0.5 * serving["achieved_particle_steps_per_s"] / work
        serving["at_sustainable_rate"] = serve_sample(args, dev, args.sustained_requests, rate=rate)
    if serving is not None and args.fifo_compare:
        f = serve_sample(args, dev, args.requests, policy="fifo")
        serving["fifo_same_stream"] = {k: f[k] for k in ("p50_latency_s", "p99_latency_s", "mean_latency_s",
                                                         "achieved_particle_steps_per_s", "max_concurrent")}
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": ensemble_config(args.sims, world, n_all),
            "details": {"sharding": "LPT over ranks by particle count, no data-path collective",
                        "sims_this_rank": len(ws), "n_particles_this_rank": n_tot,
                        "pair_split": split, "pair_kernel": pair_kernel_name(split), "graphs": True,
                        "pair_tuning": dict(zip(["split", "warps_per_cta", "grab"], tuning)),
                        "phase_ms_per_step": dict(zip(["bin", "pair", "bonded", "advance"], phase.round(5).tolist()))},
            "plain_gpu": plain, "batched_over_plain": value / plain["value"],
            "serving": serving, "workloads": workloads,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": launches_per_step() * args.steps,
        }
        print(json.dumps(line), flush=True)


def tune(eng, args):
    """Autotune the pair pass, or fix the tuple given with --tuning; returns the split."""
    if args is not None and getattr(args, "tuning", ""):
        eng.set_tuning(*(int(v) for v in args.tuning.split(",")))
        split = eng.tuning()[0]
        return split
    return eng.autotune()


def pair_kernel_name(split):
    return "k_pair_home" if split == 32 else "k_pair_tile (split %d)" % split


def measure_workload(name, dev, stream, steps, warmup, args=None):
    """One single-simulation workload at its configured size on the plain path: particle-
    steps/s over `steps` steps with the L2 flushed before each, the pair kernel's time from
    stamped steps, and its FP32 roofline fraction (algorithmic flops of the interacting pairs)."""
    import torch
    from tfg.engine import Engine, setup_model
    w = make_workload(name, 0)
    eng = Engine(w.desc(device=dev))
    keep = setup_model(eng, w)
    eng.set_stream(stream.cuda_stream)
    if w.relax_steps:
        for t in range(w.max_type):
            eng.set_type(t, 1, w.mass[t])
        eng.step(w.relax_steps)
        for t in range(w.max_type):
            eng.set_type(t, w.dynamics[t], w.mass[t])
    split = tune(eng, args)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    value = timed_rate(eng, w.n, steps, warmup, flush, stream)
    cnt, _ = eng.pair_signature()
    pairs = int(cnt.sum()) // 2
    eng.set_phase_timing(True)
    eng.step(2)
    ph = np.zeros(4)
    for _ in range(5):
        flush.zero_()
        eng.step(1)
        ph += np.array(eng.phase_ms())
    ph /= 5
    fl = pairs * pair_flops(w)
    peak = fp32_peak(dev)
    achieved = fl / (ph[1] * 1e-3) / 1e12
    del eng, keep
    return {"value": value, "unit": "particle-steps/s", "n_particles": w.n, "steps": steps,
            "ms_per_step": w.n * 1e3 / value, "description": WORKLOADS[name]["desc"],
            "l2": "flushed between timed steps (256 MiB write)",
            "roofline": {"bound": "fp32", "kernel": pair_kernel_name(split), "kernel_ms": float(ph[1]),
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None, "pairs_per_step": pairs,
                         "flops_per_pair": pair_flops(w)},
            "phase_ms_per_step": dict(zip(["bin", "pair", "bonded", "advance"], ph.round(5).tolist()))}


def run_served(args, rank, world, dev, dist):
    with ClockSampler(dev, clock_path("clocks_served.csv")) as clk:
        s = serve_sample(args, dev, args.requests or 100)
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": s["achieved_particle_steps_per_s"], "unit": "particle-steps/s",
            "n_gpus": world, "steps": s["chunks"], "warmup": 0, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "served", "description": WORKLOADS["served"]["desc"]},
            "serving": s, "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


def run_single(args, rank, world, dev, dist):
    import torch
    from tfg.engine import Engine, setup_model
    w = make_workload(args.workload, rank, args.n or None, args.relax)
    eng = Engine(w.desc(device=dev))
    keep = setup_model(eng, w)
    # a dedicated (non-default) stream shared by the engine and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    if w.relax_steps:
        # relaxation with the reference's overdamped displacement clamp (untimed)
        for t in range(w.max_type):
            eng.set_type(t, 1, w.mass[t])
        eng.step(w.relax_steps)
        for t in range(w.max_type):
            eng.set_type(t, w.dynamics[t], w.mass[t])
    split = tune(eng, args)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        eng.step(1, sync=False)
    torch.cuda.synchronize()
    cnt0, _ = eng.pair_signature()
    pairs0 = int(cnt0.sum()) // 2
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    eng.set_phase_timing(False)   # the timed steps carry no phase stamps
    eng.step(2)                   # re-capture the step graphs without them
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    rebuilds0 = eng.verlet()[0] if w.flags & 4 else 0
    with ClockSampler(dev, clock_path("clocks_bench.csv")) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            eng.step(1, sync=False)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    rebuilds1 = eng.verlet()[0] if w.flags & 4 else 0
    # phase split from stamped steps after the timed region (L2 flushed before each)
    eng.set_phase_timing(True)
    eng.step(2)
    phase_tot = np.zeros(4)
    nph = min(args.steps, 10)
    for k in range(nph):
        flush.zero_()
        eng.step(1)
        phase_tot += np.array(eng.phase_ms())
    phase_tot *= args.steps / nph
    if dist is not None:
        dist.barrier()
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    cnt1, _ = eng.pair_signature()
    pairs1 = int(cnt1.sum()) // 2
    if dist is not None:
        tt = torch.tensor([t_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    value = world * w.n * args.steps / (t_ms * 1e-3)

    # end to end: load from host arrays, run --e2e-steps steps, download
    E = args.e2e_steps or min(w.steps, 200)
    pin = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hx, hv, ht, hr, hi, hs = (pin(a) for a in (w.x, w.v, w.type, w.radius, w.imass, w.species))
    e2e_eng = Engine(w.desc(device=dev))
    keep2 = setup_model(e2e_eng, w)
    e2e_eng.set_stream(stream.cuda_stream)
    e2e_eng.set_tuning(*eng.tuning())
    ns = w.nr_species
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_eng.load(hx, v=hv, type=ht, radius=hr, imass=hi, species=hs)
    e2e_eng.step(E)
    e2e_eng.download()
    t_e2e = time.perf_counter() - t0
    bi = w.n * (12 + 12 + 4 + 4 + 4 + 4 * ns)
    bo = w.n * (12 + 12 + 4 + 12 + 12 + 4 + 8 * ns)
    e2e = {"value": world * w.n * E / t_e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": bi / E,
           "d2h_bytes_per_step": bo / E, "steps": E,
           "how": "tfg_load_particles from host arrays, tfg_step(%d), tfg_download" % E}

    pairs = 0.5 * (pairs0 + pairs1)
    fl_pair = pairs * pair_flops(w)
    pair_ms_avg = phase_tot[1] / args.steps
    achieved = fl_pair / (pair_ms_avg * 1e-3) / 1e12
    peak = fp32_peak(dev)
    step_ms = t_ms / args.steps
    bytes_alg = w.n * WORKLOADS[args.workload]["bytes_per_particle"]
    hbm, hbm_src = hbm_peak()
    roof = {"bound": "fp32", "kernel": pair_kernel_name(split), "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
            "peak_source": "measured live (tfg_probe_fp32_tflops, FFMA chains)",
            "flops_per_launch": fl_pair, "pairs_per_step": pairs, "flops_per_pair": pair_flops(w),
            "kernel_ms": pair_ms_avg, "traffic": None,
            "step_hbm": {"achieved_gbs": bytes_alg / (step_ms * 1e-3) / 1e9, "peak_gbs": hbm, "peak_source": hbm_src,
                         "frac": bytes_alg / (step_ms * 1e-3) / 1e9 / hbm, "bytes_per_step": bytes_alg}}
    verlet = None
    if w.flags & 4:   # Verlet mode: the same fluid with cell lists, and Verlet without pair lists
        rb_timed = rebuilds1 - rebuilds0
        wc = make_workload("lj_fluid", rank, args.n or None)
        cmp = {}
        for label, ww, lists in (("cell_lists", wc, True), ("verlet_without_pair_lists", w, False)):
            e = Engine(ww.desc(device=dev))
            k = setup_model(e, ww)
            e.set_stream(stream.cuda_stream)
            e.set_pair_lists(lists)
            cmp[label] = timed_rate(e, ww.n, args.steps, args.warmup, flush, stream, world)
            del e, k
        verlet = {"skin": float(min(d / c for d, c in zip(w.dim, w.cells)) - w.cutoff),
                  "rebuilds_in_timed_steps": rb_timed, "steps": args.steps,
                  "cell_lists_value": cmp["cell_lists"], "verlet_without_pair_lists_value": cmp["verlet_without_pair_lists"],
                  "speedup_over_cell_lists": value / cmp["cell_lists"],
                  "how": "same fluid, same steps and L2 flush; cell lists at cell edge >= cutoff"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, steps, dt = cpu_rate_sims([w], threads, 15.0, max_steps=100)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": "%d steps of the %s workload (%d particles) on the threaded CPU restatement "
                         "of the reference engine, %.1f s" % (steps[0], args.workload, w.n, dt)}
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload]["desc"],
                       "n_particles": w.n, "cells": list(w.cells), "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": "replicas%d" % world, "pair_split": split,
                       "phase_ms_per_step": dict(zip(["bin", "pair", "bonded", "advance"],
                                                     (phase_tot / args.steps).round(5).tolist()))},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
            "gpu_launches": launches_per_step(w.bonds is not None, w.angles is not None) * args.steps,
        }
        if verlet:
            line["verlet"] = verlet
        print(json.dumps(line), flush=True)
    del keep, keep2


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="ensemble", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="tfg", choices=["tfg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end job (0: the workload's own step count, 1,000 for the ensemble)")
    ap.add_argument("--sustained-requests", type=int, default=40,
                    help="served requests at a sustainable arrival rate (0: skip)")
    ap.add_argument("--n", type=int, default=0, help="scale a single-simulation workload to n particles")
    ap.add_argument("--relax", type=int, default=None, help="override the relaxation steps")
    ap.add_argument("--sims", type=int, default=256, help="simulations in the ensemble")
    ap.add_argument("--plain-steps", type=int, default=20, help="timed steps per simulation on the plain path")
    ap.add_argument("--requests", type=int, default=100, help="served-stream sample size (0: skip)")
    ap.add_argument("--fifo-compare", type=int, default=1,
                    help="also serve the sample first-come-first-served, for comparison (0: skip)")
    ap.add_argument("--serve-particles", type=int, default=2_000_000, help="particles in flight cap")
    ap.add_argument("--quantum", type=int, default=50, help="largest chunk of steps between admissions")
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--sub-workloads", default="bonded_fluid,dpd_droplets,dpd_droplets_species",
                    help="single-simulation workloads measured beside the ensemble (comma list; empty: none)")
    ap.add_argument("--sub-steps", type=int, default=40, help="timed steps of each of those workloads")
    ap.add_argument("--tuning", default="", help="fix the pair pass's tuple 'split,warps,grab' instead of autotuning")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_reference(args, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.build()
    if args.workload == "ensemble":
        run_ensemble(args, rank, world, dev, dist)
    elif args.workload == "served":
        run_served(args, rank, world, dev, dist)
    else:
        run_single(args, rank, world, dev, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
