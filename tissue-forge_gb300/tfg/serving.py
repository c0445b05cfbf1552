"""Continuous batching of simulation requests on one GPU.

A request is an independent simulation (a configs.Workload) to be advanced a given number
of steps; its result is the final particle state.  The server keeps one batch (a device
arena, tfg_batch_*) per model family -- simulations of one batch share their type count
and species count -- and every batch runs on its own CUDA stream, so the families' steps
overlap on the device.

Admission runs under two limits: an HBM byte budget (the arena footprint of a simulation,
estimated per particle and per cell) and a cap on particles in flight (past the point where
the GPU is full, more simulations only share it more thinly and every latency grows).  Among
the requests that have arrived, the default policy admits the least work first (particles x
steps), so that a short request does not wait behind long ones that share the GPU; the
"fifo" policy admits in arrival order.  A batch advances in chunks of at most `quantum` steps, cut
short so that no simulation runs past its step count.  At a chunk boundary the finished
simulations are downloaded and removed; requests that arrived meanwhile were already
added (host-side) and join at the next chunk, without waiting for the batch to drain.
Latency is completion time minus arrival time.
"""
import collections
import heapq
import time

import numpy as np

from .engine import Batch, setup_model

# Device bytes per particle of an arena: two particle buffers (pos, vel, aux, fext,
# pforce float4; cell int32; value and increment per species), the force buffer and the
# binning scratch (five int32 arrays).
def _bytes_per_particle(nspec):
    return 2 * (5 * 16 + 4 + 8 * max(1, nspec)) + 16 + 5 * 4


def footprint(w):
    """Estimated arena bytes of one simulation (particles, cells, bonds, angles)."""
    nb = 0 if w.bonds is None else len(w.bonds)
    na = 0 if w.angles is None else len(w.angles)
    return (w.n * _bytes_per_particle(w.nr_species) + int(np.prod(w.cells)) * 16 + 12 * 3 * max(w.cells)
            + nb * 12 + na * 16)


class Request:
    __slots__ = ("rid", "t_arrival", "workload", "steps", "t_admit", "t_done", "result", "reductions")

    def __init__(self, rid, t_arrival, workload, steps):
        self.rid = rid
        self.t_arrival = float(t_arrival)
        self.workload = workload
        self.steps = int(steps)
        self.t_admit = None
        self.t_done = None
        self.result = None
        self.reductions = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival


class _Active:
    __slots__ = ("req", "sim", "remaining", "keep")

    def __init__(self, req, sim, keep):
        self.req = req
        self.sim = sim
        self.remaining = req.steps
        self.keep = keep


class Lane:
    """One model family: a Batch on its own stream and its active simulations."""

    def __init__(self, max_type, nspec, device=0, batch=None):
        self.batch = batch if batch is not None else Batch(max_type, nspec, device)
        self.active = {}
        self.running = 0
        self.in_chunk = set()
        self.pot_cache = {}

    def admit(self, req):
        w = req.workload
        sim = self.batch.add_sim(w.desc())
        keep = setup_model(sim, w, pot_cache=self.pot_cache)
        self.active[sim.sid] = _Active(req, sim, keep)

    def launch(self, quantum):
        chunk = min(quantum, min(a.remaining for a in self.active.values()))
        self.batch.step(chunk, sync=False)
        self.running = chunk
        # simulations admitted while this chunk runs join the next one
        self.in_chunk = set(self.active)

    def idle(self):
        return self.batch.idle()

    def finish_chunk(self, clock, keep_results=True):
        """Account the chunk just completed; download and retire the finished simulations.
        Returns the requests that completed."""
        self.batch.sync()
        done = []
        for sid in self.in_chunk:
            a = self.active[sid]
            a.remaining -= self.running
            if a.remaining == 0:
                done.append(a)
        self.running = 0
        for a in done:
            if keep_results:
                a.req.result = a.sim.download()
                a.req.reductions = a.sim.reductions()
            a.req.t_done = clock()
        for a in done:
            self.batch.remove_sim(a.sim)
            del self.active[a.sim.sid]
        return [a.req for a in done]

    def particles(self):
        return sum(a.req.workload.n for a in self.active.values())


class Server:
    """Continuous-batching request loop over one GPU (see the module docstring)."""

    def __init__(self, budget_bytes=150 << 30, max_particles=2_000_000, quantum=50, device=0,
                 keep_results=True, lane_factory=None, policy="sjf"):
        if policy not in ("sjf", "fifo"):
            raise ValueError("policy is 'sjf' or 'fifo'")
        self.policy = policy
        self.budget = int(budget_bytes)
        self.max_particles = int(max_particles)
        self.quantum = int(quantum)
        self.device = device
        self.keep_results = keep_results
        self.lane_factory = lane_factory or (lambda max_type, nspec: Lane(max_type, nspec, device))
        self.lanes = {}
        self.bytes_in_flight = 0
        self.particles_in_flight = 0
        self.max_concurrent = 0
        self.chunks = 0

    def _lane(self, w):
        key = (w.max_type, w.nr_species)
        if key not in self.lanes:
            self.lanes[key] = self.lane_factory(w.max_type, w.nr_species)
        return self.lanes[key]

    def _fits(self, w):
        if self.bytes_in_flight + footprint(w) > self.budget:
            return False
        return self.particles_in_flight == 0 or self.particles_in_flight + w.n <= self.max_particles

    def run(self, requests, clock=None, sleep=time.sleep):
        """Serve `requests` (arrival times in seconds from the start).  Returns them, each
        with t_admit, t_done, result and reductions filled in."""
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrival))
        for r in pending:
            if footprint(r.workload) > self.budget:
                raise ValueError("request %r does not fit the HBM budget" % r.rid)
        t0 = time.perf_counter()
        clock = clock or (lambda: time.perf_counter() - t0)
        finished = []
        total = len(pending)
        arrived = []   # heap of (priority, arrival, id, request)
        while len(finished) < total:
            now = clock()
            while pending and pending[0].t_arrival <= now:
                r = pending.popleft()
                key = r.workload.n * r.steps if self.policy == "sjf" else 0
                heapq.heappush(arrived, (key, r.t_arrival, r.rid, r))
            while arrived and self._fits(arrived[0][3].workload):
                r = heapq.heappop(arrived)[3]
                self._lane(r.workload).admit(r)
                r.t_admit = clock()
                self.bytes_in_flight += footprint(r.workload)
                self.particles_in_flight += r.workload.n
            live = sum(len(l.active) for l in self.lanes.values())
            self.max_concurrent = max(self.max_concurrent, live)
            for lane in self.lanes.values():
                if lane.running == 0 and lane.active:
                    lane.launch(self.quantum)
                    self.chunks += 1
            running = [l for l in self.lanes.values() if l.running]
            if not running:
                if pending:
                    sleep(max(0.0, min(0.01, pending[0].t_arrival - clock())))
                elif arrived and not any(l.active for l in self.lanes.values()):
                    raise RuntimeError("request %r cannot be admitted" % arrived[0][3].rid)
                continue
            progressed = False
            for lane in running:
                if lane.idle():
                    for r in lane.finish_chunk(clock, self.keep_results):
                        finished.append(r)
                        self.bytes_in_flight -= footprint(r.workload)
                        self.particles_in_flight -= r.workload.n
                    progressed = True
            if not progressed:
                sleep(0.0002)
        return finished


def summarize(reqs):
    """Throughput and latency figures of a served run."""
    lat = np.array([r.latency for r in reqs], np.float64)
    work = float(sum(r.workload.n * r.steps for r in reqs))
    t_first = min(r.t_arrival for r in reqs)
    t_last = max(r.t_done for r in reqs)
    span_arrivals = max(r.t_arrival for r in reqs) - t_first
    return {
        "requests": len(reqs),
        "particle_steps": work,
        "makespan_s": t_last - t_first,
        "achieved_particle_steps_per_s": work / max(t_last - t_first, 1e-9),
        "offered_particle_steps_per_s": work / span_arrivals if span_arrivals > 0 else None,
        "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)),
        "mean_latency_s": float(lat.mean()),
    }
