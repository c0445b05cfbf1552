"""Benchmark of the per-step particle path: particle-steps/s on one GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl tfg|reference]

A "step" is one full engine step (re-bin, fused pair pass, bonded, advance, reductions)
over one simulation held resident in HBM.  The default workload is the DPD-droplets
configuration (100,000 particles, box 40, cutoff 1, DPD + Fickian flux).  Between timed
steps the L2 is flushed by writing a 256 MiB buffer (the working set is smaller than L2).

value  = particle-steps/s with state resident on the device (CUDA events on the engine's
         stream, summed over the K timed steps, max over ranks).
e2e    = the same metric through the reference-facing C ABI with host buffers: every step
         uploads the particle state from pinned host memory (tfg_load_particles_binned),
         runs one step and downloads positions, velocities and species (tfg_download).
roofline: the pair kernel against the measured FP32 FMA peak (tfg_probe_fp32_tflops).
cpu_baseline: the CPU restatement of the reference engine (threaded, all host cores) on a
         bounded sample of the same workload.
--impl reference: the CPU restatement of the reference engine timed on the host cores (the
         reference itself cannot be built: its Magnum/Corrade/libsbml submodules are empty
         and it needs GL/GLFW/assimp).
For N>1 (torchrun) every rank runs an independent replica of the workload (the path has no
data-path exchange between simulations): scaling "weak", value = all ranks' particle-steps
divided by the slowest rank's time.
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
    "dpd_droplets": dict(desc="DPD droplets with Fickian flux: 100,000 particles, box 40, cutoff 1, "
                              "alpha 10 gamma 4.5 sigma 3, Fick k 0.5, dt 0.01", bytes_per_particle=88),
    "bonded_fluid": dict(desc="LJ 12-6 fluid in chains of 16 with harmonic bonds and angles: 2,000,000 particles "
                              "at density 0.85, cutoff 2.5, dt 0.002", bytes_per_particle=80),
    "cell_sorting": dict(desc="cell sorting: 4,000 particles, box 20, cutoff 3, shifted Morse, overdamped",
                         bytes_per_particle=48),
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
    if name == "bonded_fluid":
        w = configs.bonded_fluid(n=n or 2_000_000, seed=2 + seed)
        if relax is not None:
            w.relax_steps = relax
        return w
    if name == "cell_sorting":
        if n:
            return configs.cell_sorting(n=n, side=20.0 * (n / 4000) ** (1.0 / 3.0), seed=seed)
        return configs.cell_sorting(seed=seed)
    raise SystemExit("unknown workload " + name)


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


def run_reference(args, rank, world):
    if rank != 0:
        return
    w = make_workload(args.workload, 0, args.n or None, args.relax)
    threads = os.cpu_count() or 1
    budget = 20.0
    rates = []
    for k in range(args.warmup + args.steps):
        rate, steps, dt = cpu_reference_rate(w, threads, budget / max(1, args.steps), max_steps=50)
        if k >= args.warmup:
            rates.append((rate, steps, dt))
    total_ps = sum(r[1] for r in rates) * w.n
    total_t = sum(r[2] for r in rates)
    value = total_ps / total_t
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / max(1, sum(r[1] for r in rates)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload]["desc"], "n_particles": w.n},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": "%d engine steps of the %s workload per timed step, threaded oracle "
                                   "(CPU restatement of the reference engine)" % (rates[0][1], args.workload)},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="dpd_droplets", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="tfg", choices=["tfg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--n", type=int, default=0, help="scale the workload to n particles (same density)")
    ap.add_argument("--relax", type=int, default=None, help="override the relaxation steps")
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
    import ctypes as C
    from tfg import lib
    from tfg.engine import Engine, setup_model

    w = make_workload(args.workload, rank, args.n or None, args.relax)
    eng = Engine(w.desc(device=dev))
    keep = setup_model(eng, w)
    # a dedicated (non-default) stream shared by the engine and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    if w.relax_steps:
        # steepest-descent-like relaxation with the reference's displacement clamp (untimed)
        for t in range(w.max_type):
            eng.set_type(t, 1, w.mass[t])
        eng.step(w.relax_steps)
        for t in range(w.max_type):
            eng.set_type(t, w.dynamics[t], w.mass[t])

    split = eng.autotune()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        eng.step(1, sync=False)
    torch.cuda.synchronize()
    cnt0, _ = eng.pair_signature()
    pairs0 = int(cnt0.sum()) // 2

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    pair_ms = 0.0
    phase_tot = np.zeros(4)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev, os.path.join(ROOT, "gpurun_out", "clocks_bench.csv") if os.path.isdir(
            os.path.join(ROOT, "gpurun_out")) else "/tmp/clocks_bench.csv") as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            eng.step(1, sync=False)
            ev[k][1].record(stream)
            ph = eng.phase_ms()
            phase_tot += np.array(ph)
        torch.cuda.synchronize()
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

    # ---- end-to-end through the C ABI with host buffers
    e2e = None
    out = eng.download()
    cell, xrel = out["cell"], out["xrel"]
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h_cell, h_xrel, h_v = pin(cell), pin(xrel), pin(out["v"])
    h_type, h_rad, h_im = pin(w.type), pin(w.radius), pin(w.imass)
    h_sp = pin(out["species"]) if w.nr_species else None
    e2e_eng = Engine(w.desc(device=dev))
    keep2 = setup_model(e2e_eng, w)
    ns = w.nr_species
    bi = w.n * (4 + 12 + 12 + 4 + 4 + 4 + 4 * ns)
    bo = w.n * (12 + 12 + 4 + 4 * ns)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        e2e_eng.load_binned(h_cell, h_xrel, v=h_v, type=h_type, radius=h_rad, imass=h_im, species=h_sp)
        e2e_eng.step(1, sync=True)
        o = e2e_eng.download()
        h_cell, h_xrel, h_v = o["cell"], o["xrel"], o["v"]
        if ns:
            h_sp = o["species"]
    t_e2e = time.perf_counter() - t0
    e2e = {"value": w.n * args.e2e_steps / t_e2e * world, "unit": "particle-steps/s",
           "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo, "steps": args.e2e_steps}

    # ---- roofline of the pair kernel
    pairs = 0.5 * (pairs0 + pairs1)
    fl_pair = pairs * pair_flops(w)
    pair_ms_avg = phase_tot[1] / args.steps
    achieved = fl_pair / (pair_ms_avg * 1e-3) / 1e12
    peak = C.c_double(0.0)
    lib().tfg_probe_fp32_tflops(dev, C.byref(peak))
    step_ms = t_ms / args.steps
    bytes_alg = w.n * WORKLOADS[args.workload]["bytes_per_particle"]
    hbm = None
    try:
        hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        hbm = 6800.0
    roof = {"bound": "fp32", "kernel": "k_pair_tile (split %d)" % split, "achieved": achieved, "peak": peak.value,
            "unit": "TFLOP/s", "frac": achieved / peak.value if peak.value else None,
            "peak_source": "measured live (tfg_probe_fp32_tflops, FFMA chains)",
            "flops_per_launch": fl_pair, "pairs_per_step": pairs, "flops_per_pair": pair_flops(w),
            "kernel_ms": pair_ms_avg, "traffic": None,
            "step_hbm": {"achieved_gbs": bytes_alg / (step_ms * 1e-3) / 1e9, "peak_gbs": hbm,
                         "frac": bytes_alg / (step_ms * 1e-3) / 1e9 / hbm, "bytes_per_step": bytes_alg}}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, steps, dt = cpu_reference_rate(w, threads, 15.0, max_steps=100)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": "%d steps of the %s workload (%d particles) on the threaded CPU restatement "
                         "of the reference engine, %.1f s" % (steps, args.workload, w.n, dt)}

    launches_per_step = 9 + (1 if w.bonds is not None else 0) + (1 if w.angles is not None else 0)
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
            "gpu_launches": launches_per_step * args.steps,
        }
        print(json.dumps(line), flush=True)
    del keep, keep2
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
