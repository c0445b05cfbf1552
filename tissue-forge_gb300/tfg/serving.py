"""Continuous batching of simulation requests on one GPU: the Python client of the
library's server (tfg_server_*, tfg_request_* in include/tfg.h).

A request is an independent simulation (a configs.Workload) to be advanced a given number
of steps; its result is the final particle state.  The server itself is native: it keeps
one batch (a device arena, tfg_batch_*) per model family -- simulations of one batch share
their type count and species count -- on its own CUDA stream, admits arrived requests under
an HBM byte budget and a cap on particles in flight (least work, particles x steps, first;
or first come, first served), advances every batch in chunks of at most `quantum` steps (a
simulation that reaches its step count inside a chunk stops itself there and waits,
unchanged, for the chunk to end), and at each chunk boundary retires the finished
simulations and admits waiting requests, which join without waiting for the batch to
drain.  A simulation whose particles raise an error (non-finite position, a particle
faster than one cell per step) is retired as failed with that status while the rest of its
batch continues.  This module builds each request through the C ABI (RequestBuilder has the
engine-like method names, so engine.setup_model fills it), submits it at its arrival time and
drives the loop with tfg_server_poll.  Latency is completion time minus arrival time.
"""
import collections
import ctypes as C
import time

import numpy as np

from . import abi
from ._lib import lib as _default_lib
from .engine import setup_model


def _bytes_per_particle(nspec):
    # two particle buffers (pos, vel, aux, fext, pforce float4; cell int32; value and
    # increment per species), the force buffer and the binning scratch (five int32 arrays)
    return 2 * (5 * 16 + 4 + 8 * max(1, nspec)) + 16 + 5 * 4


def footprint(w):
    """Arena bytes of one simulation as the server estimates them (particles, cells, bonds,
    angles)."""
    nb = 0 if w.bonds is None else len(w.bonds)
    na = 0 if w.angles is None else len(w.angles)
    return w.n * _bytes_per_particle(w.nr_species) + int(np.prod(w.cells)) * 16 + nb * 12 + na * 16


class _Shape:
    """What the client keeps of a lazily built request's workload once it is submitted."""
    __slots__ = ("n", "nr_species", "name")

    def __init__(self, w):
        self.n, self.nr_species, self.name = w.n, w.nr_species, w.name


class Request:
    """One simulation request.  `workload` is a configs.Workload, or None with `make` a
    callable that builds it: such a request is built when it arrives, and after submission
    the client keeps only its shape (the server holds the particle data)."""
    __slots__ = ("rid", "t_arrival", "workload", "steps", "t_admit", "t_done", "result", "reductions", "status",
                 "make", "t_admit_server")

    def __init__(self, rid, t_arrival, workload, steps, make=None):
        self.rid = rid
        self.t_arrival = float(t_arrival)
        self.workload = workload
        self.make = make
        self.steps = int(steps)
        self.t_admit = None
        self.t_admit_server = None   # admission time on the server's own clock (orders admissions)
        self.t_done = None
        self.result = None
        self.reductions = None
        self.status = None   # 0 when finished, a TFG_E_* code when retired as failed

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival


def _fp(a):
    return None if a is None else a.ctypes.data_as(abi.F_P)


def _ip(a):
    return None if a is None else a.ctypes.data_as(abi.I_P)


def _up(a):
    return None if a is None else a.ctypes.data_as(abi.U_P)


def _conv(a, dt):
    return None if a is None else np.ascontiguousarray(a, dt)


class RequestBuilder:
    """One request recorded through tfg_request_*; the method names are an engine's."""

    def __init__(self, L, w, steps):
        self.L = L
        self.h = C.c_void_p()
        desc = w.desc()
        self._chk(L.tfg_request_create(C.byref(desc), w.max_type, w.nr_species, int(steps), C.byref(self.h)),
                  "request_create")

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: %s" % (what, abi.STATUS_NAMES.get(rc, rc)))

    def free(self):
        if self.h:
            self.L.tfg_request_free(self.h)
            self.h = C.c_void_p()

    def set_type(self, t, dynamics, mass=1.0):
        self._chk(self.L.tfg_request_set_type(self.h, t, dynamics, mass), "request_set_type")

    def set_potential(self, ti, tj, ptr):
        self._chk(self.L.tfg_request_set_potential(self.h, ti, tj, ptr), "request_set_potential")

    def add_flux(self, ti, tj, flux):
        self._chk(self.L.tfg_request_add_flux(self.h, ti, tj, C.byref(flux)), "request_add_flux")

    def set_species_flags(self, flags):
        a = np.ascontiguousarray(flags, np.uint32)
        self._chk(self.L.tfg_request_set_species_flags(self.h, len(a), _up(a)), "request_set_species_flags")

    def set_random_force(self, t, mean, std, duration_steps):
        self._chk(self.L.tfg_request_set_random_force(self.h, t, mean, std, duration_steps),
                  "request_set_random_force")

    def set_species_reset(self, values):
        a = np.ascontiguousarray(values, np.float32)
        self._chk(self.L.tfg_request_set_species_reset(self.h, len(a), _fp(a)), "request_set_species_reset")

    def set_boundary(self, wall, kind, velocity=(0.0, 0.0, 0.0), restore=1.0, radius=0.0):
        b = abi.boundary(kind, velocity, restore, radius)
        self._chk(self.L.tfg_request_set_boundary(self.h, wall, C.byref(b)), "request_set_boundary")

    def set_boundary_potential(self, wall, t, ptr):
        self._chk(self.L.tfg_request_set_boundary_potential(self.h, wall, t, ptr), "request_set_boundary_potential")

    def set_bonded_potential(self, slot, ptr):
        self._chk(self.L.tfg_request_set_bonded_potential(self.h, slot, ptr), "request_set_bonded_potential")

    def load(self, x, v=None, type=None, radius=None, imass=None, flags=None, species=None, force_i=None):
        x = np.ascontiguousarray(x, np.float32)
        v, radius, imass, species, force_i = (_conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = _conv(type, np.int32)
        flags = _conv(flags, np.uint32)
        self._chk(self.L.tfg_request_load_particles(self.h, x.shape[0], _fp(x), _fp(v), _ip(type), _fp(radius),
                                                    _fp(imass), _up(flags), _fp(species), _fp(force_i)),
                  "request_load_particles")

    def load_bonds(self, i, j, slot=None):
        i, j = (np.ascontiguousarray(a, np.int32) for a in (i, j))
        slot = _conv(slot, np.int32)
        self._chk(self.L.tfg_request_load_bonds(self.h, len(i), _ip(i), _ip(j), _ip(slot)), "request_load_bonds")

    def load_angles(self, i, j, k, slot=None):
        i, j, k = (np.ascontiguousarray(a, np.int32) for a in (i, j, k))
        slot = _conv(slot, np.int32)
        self._chk(self.L.tfg_request_load_angles(self.h, len(i), _ip(i), _ip(j), _ip(k), _ip(slot)),
                  "request_load_angles")


class Server:
    """The native request loop (see the module docstring).  `lib` is the library that
    provides tfg_server_* (the product's by default)."""

    def __init__(self, budget_bytes=150 << 30, max_particles=2_000_000, quantum=50, device=0,
                 keep_results=True, policy="sjf", lib=None):
        if policy not in ("sjf", "fifo"):
            raise ValueError("policy is 'sjf' or 'fifo'")
        self.L = lib if lib is not None else _default_lib()
        self.policy = policy
        self.budget = int(budget_bytes)
        self.keep_results = keep_results
        d = abi.ServerDesc()
        d.device = device
        d.quantum = int(quantum)
        d.budget_bytes = self.budget
        d.max_particles = int(max_particles)
        d.policy = abi.SERVER_LEAST_WORK if policy == "sjf" else abi.SERVER_FIFO
        d.discard_results = 0 if keep_results else 1
        self.h = C.c_void_p()
        rc = self.L.tfg_server_create(C.byref(d), C.byref(self.h))
        if rc != 0:
            raise RuntimeError("tfg_server_create failed: %s" % abi.STATUS_NAMES.get(rc, rc))
        self._pots = []   # product potentials the recorded requests were built from

    def close(self):
        if self.h:
            self.L.tfg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        st = abi.ServerStats()
        self.L.tfg_server_get_stats(self.h, C.byref(st))
        return {k: (float if t is C.c_double else int)(getattr(st, k)) for k, t in abi.ServerStats._fields_}

    @property
    def max_concurrent(self):
        return self.stats()["max_concurrent"]

    @property
    def chunks(self):
        return self.stats()["chunks"]

    def _submit(self, r, pot_cache):
        if r.workload is None:
            r.workload = r.make()
        if footprint(r.workload) > self.budget:
            raise ValueError("request %r does not fit the HBM budget" % r.rid)
        b = RequestBuilder(self.L, r.workload, r.steps)
        try:
            self._pots.extend(setup_model(b, r.workload, pot_cache=pot_cache))
        except Exception:
            b.free()
            raise
        rid = C.c_int64()
        rc = self.L.tfg_server_submit(self.h, b.h, C.byref(rid))
        if rc != 0:
            b.free()
            raise RuntimeError("tfg_server_submit: %s (%s)" % (abi.STATUS_NAMES.get(rc, rc),
                                                              self.L.tfg_server_last_error(self.h).decode()))
        b.h = C.c_void_p()   # the server owns it now
        if r.make is not None:
            r.workload = _Shape(r.workload)
        return int(rid.value)

    def _collect(self, sid, r, now, t_submit):
        """Fill r from the server's record of request sid; the server's admission time is
        mapped onto this clock through the submission time seen on both clocks."""
        state, status = C.c_int(), C.c_int()
        t = (C.c_double * 3)()
        self.L.tfg_server_request_info(self.h, sid, C.byref(state), C.byref(status), t)
        r.t_done = now
        r.t_admit = max(r.t_arrival, t_submit + (t[1] - t[0])) if t[1] >= 0 else None
        r.t_admit_server = t[1] if t[1] >= 0 else None
        r.status = int(status.value)
        if state.value == abi.REQ_DONE and self.keep_results:
            n = C.c_int()
            self.L.tfg_server_result(self.h, sid, C.byref(n), None, None, None, None)
            n = int(n.value)
            ns = r.workload.nr_species
            out = dict(x=np.zeros((n, 3), np.float32), v=np.zeros((n, 3), np.float32),
                       species=np.zeros((n, ns), np.float32))
            red = abi.Reductions()
            self.L.tfg_server_result(self.h, sid, None, _fp(out["x"]), _fp(out["v"]),
                                     _fp(out["species"]) if ns else None, C.byref(red))
            r.result, r.reductions = out, red
        self.L.tfg_server_release(self.h, sid)

    def run(self, requests, clock=None, sleep=time.sleep):
        """Serve `requests` (arrival times in seconds from the start): each is submitted at its
        arrival time.  Returns them, each with t_admit, t_done, status, result and reductions
        filled in (result None for a failed request)."""
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrival))
        for r in pending:
            if r.workload is not None and footprint(r.workload) > self.budget:
                raise ValueError("request %r does not fit the HBM budget" % r.rid)
        t0 = time.perf_counter()
        clock = clock or (lambda: time.perf_counter() - t0)
        pot_cache = {}
        by_id = {}
        finished = []
        total = len(pending)
        ids = (C.c_int64 * 256)()
        got = C.c_int()
        done = C.c_int()
        while len(finished) < total:
            now = clock()
            while pending and pending[0].t_arrival <= now:
                r = pending.popleft()
                sid = self._submit(r, pot_cache)
                by_id[sid] = (r, clock())
            st = self.stats()
            wait_us = 2000 if st["running"] else 0
            rc = self.L.tfg_server_poll(self.h, wait_us, C.byref(done))
            if rc != 0:
                raise RuntimeError("tfg_server_poll: %s (%s)" % (abi.STATUS_NAMES.get(rc, rc),
                                                                self.L.tfg_server_last_error(self.h).decode()))
            while True:
                self.L.tfg_server_take_finished(self.h, ids, len(ids), C.byref(got))
                if got.value == 0:
                    break
                t = clock()
                for k in range(got.value):
                    sid = int(ids[k])
                    r, t_submit = by_id.pop(sid)
                    self._collect(sid, r, t, t_submit)
                    finished.append(r)
            if not self.stats()["running"] and len(finished) < total:
                if pending:
                    sleep(max(0.0, min(0.01, pending[0].t_arrival - clock())))
                elif not by_id:
                    break
                elif self.stats()["queued"] and not self.stats()["running"]:
                    raise RuntimeError("a request cannot be admitted")
        return finished


def backlogged_rate(reqs):
    """Particle-steps per second while requests were waiting for admission: from the first
    admission to the last, each finished request's particle-steps spread evenly over its
    time in the server.  This is the served rate without the start of the run (filling the
    server) and its drain (the last requests running with room to spare).  None when every
    request was admitted at once."""
    ok = [r for r in reqs if not r.status and r.t_admit is not None and r.t_done > r.t_admit]
    if not ok:
        return None
    t0, t1 = min(r.t_admit for r in ok), max(r.t_admit for r in ok)
    if t1 - t0 <= 0:
        return None
    acc = 0.0
    for r in ok:
        lo, hi = max(r.t_admit, t0), min(r.t_done, t1)
        if hi > lo:
            acc += r.workload.n * r.steps * (hi - lo) / (r.t_done - r.t_admit)
    return acc / (t1 - t0)


def summarize(reqs):
    """Throughput and latency figures of a served run (failed requests count in latency,
    not in the particle-steps)."""
    lat = np.array([r.latency for r in reqs], np.float64)
    work = float(sum(r.workload.n * r.steps for r in reqs if not r.status))
    t_first = min(r.t_arrival for r in reqs)
    t_last = max(r.t_done for r in reqs)
    span_arrivals = max(r.t_arrival for r in reqs) - t_first
    return {
        "backlogged_particle_steps_per_s": backlogged_rate(reqs),
        "requests": len(reqs),
        "failed": sum(1 for r in reqs if r.status),
        "particle_steps": work,
        "makespan_s": t_last - t_first,
        "achieved_particle_steps_per_s": work / max(t_last - t_first, 1e-9),
        "offered_particle_steps_per_s": work / span_arrivals if span_arrivals > 0 else None,
        "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)),
        "mean_latency_s": float(lat.mean()),
    }
