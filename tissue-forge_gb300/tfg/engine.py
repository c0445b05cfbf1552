"""Python handle of one GB300 engine (libtfg's tfg_engine).

Method names mirror the reference engine's operations: set_potential ~ engine_addpot
(tfEngine.cpp:1054), add_flux ~ engine_addfluxes (:1079), load ~ space_addpart
(tfSpace.cpp:477), step ~ engine_step (:1378), force_only ~ engine_force_prep +
engine_force (:1431-1557).
"""
import ctypes as C

import numpy as np

from . import abi
from ._lib import lib
from .potentials import Potential


class TfgError(RuntimeError):
    def __init__(self, code, what, msg=""):
        super().__init__("%s failed: %s %s" % (what, abi.STATUS_NAMES.get(code, code), msg))
        self.code = code


def _fp(a):
    return None if a is None else a.ctypes.data_as(abi.F_P)


def _ip(a):
    return None if a is None else a.ctypes.data_as(abi.I_P)


def _up(a):
    return None if a is None else a.ctypes.data_as(abi.U_P)


def _conv(a, dt):
    return None if a is None else np.ascontiguousarray(a, dt)


class Engine:
    def __init__(self, desc):
        self.L = lib()
        self.h = C.c_void_p()
        self.desc = desc
        self.nspec = desc.nr_species
        rc = self.L.tfg_engine_create(C.byref(desc), C.byref(self.h))
        if rc != 0:
            raise TfgError(rc, "tfg_engine_create")
        self.n = 0
        self._keep = []

    def _chk(self, rc, what):
        if rc != 0:
            raise TfgError(rc, what, self.L.tfg_last_error(self.h).decode(errors="replace"))

    def close(self):
        if self.h:
            self.L.tfg_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_type(self, t, dynamics, mass=1.0):
        self._chk(self.L.tfg_set_type(self.h, t, dynamics, mass), "set_type")

    def set_potential(self, ti, tj, pot):
        ptr = pot.ptr if isinstance(pot, Potential) else pot
        self._chk(self.L.tfg_set_potential(self.h, ti, tj, ptr), "set_potential")

    def add_flux(self, ti, tj, flux):
        self._chk(self.L.tfg_add_flux(self.h, ti, tj, C.byref(flux)), "add_flux")

    def set_species_flags(self, flags):
        a = np.ascontiguousarray(flags, np.uint32)
        self._chk(self.L.tfg_set_species_flags(self.h, len(a), _up(a)), "set_species_flags")

    def set_species_reset(self, values):
        a = np.ascontiguousarray(values, np.float32)
        self._chk(self.L.tfg_set_species_reset(self.h, len(a), _fp(a)), "set_species_reset")

    def set_stop(self, step):
        """Stop at clock `step` (-1: run on); later steps leave the simulation as it is."""
        self._chk(self.L.tfg_set_stop(self.h, int(step)), "set_stop")

    def set_random_force(self, t, mean, std, duration_steps):
        self._chk(self.L.tfg_set_random_force(self.h, t, mean, std, duration_steps), "set_random_force")

    def set_bonded_potential(self, slot, pot):
        ptr = pot.ptr if isinstance(pot, Potential) else pot
        self._chk(self.L.tfg_set_bonded_potential(self.h, slot, ptr), "set_bonded_potential")

    def set_boundary(self, wall, kind, velocity=(0.0, 0.0, 0.0), restore=1.0, radius=0.0):
        b = abi.boundary(kind, velocity, restore, radius)
        self._chk(self.L.tfg_set_boundary(self.h, wall, C.byref(b)), "set_boundary")

    def set_boundary_potential(self, wall, t, pot):
        ptr = pot.ptr if isinstance(pot, Potential) else pot
        self._chk(self.L.tfg_set_boundary_potential(self.h, wall, t, ptr), "set_boundary_potential")

    def load(self, x, v=None, type=None, radius=None, imass=None, flags=None, species=None, force_i=None):
        x = np.ascontiguousarray(x, np.float32)
        self.n = x.shape[0]
        v, radius, imass, species, force_i = (_conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = _conv(type, np.int32)
        flags = _conv(flags, np.uint32)
        self._chk(self.L.tfg_load_particles(self.h, self.n, _fp(x), _fp(v), _ip(type), _fp(radius), _fp(imass),
                                            _up(flags), _fp(species), _fp(force_i)), "load_particles")

    def load_binned(self, cell, xrel, v=None, type=None, radius=None, imass=None, flags=None, species=None,
                    force_i=None):
        cell = np.ascontiguousarray(cell, np.int32)
        xrel = np.ascontiguousarray(xrel, np.float32)
        self.n = cell.shape[0]
        v, radius, imass, species, force_i = (_conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = _conv(type, np.int32)
        flags = _conv(flags, np.uint32)
        self._chk(self.L.tfg_load_particles_binned(self.h, self.n, _ip(cell), _fp(xrel), _fp(v), _ip(type),
                                                   _fp(radius), _fp(imass), _up(flags), _fp(species),
                                                   _fp(force_i)), "load_particles_binned")

    def load_bonds(self, i, j, slot=None):
        i, j = (np.ascontiguousarray(a, np.int32) for a in (i, j))
        slot = _conv(slot, np.int32)
        self._chk(self.L.tfg_load_bonds(self.h, len(i), _ip(i), _ip(j), _ip(slot)), "load_bonds")

    def load_angles(self, i, j, k, slot=None):
        i, j, k = (np.ascontiguousarray(a, np.int32) for a in (i, j, k))
        slot = _conv(slot, np.int32)
        self._chk(self.L.tfg_load_angles(self.h, len(i), _ip(i), _ip(j), _ip(k), _ip(slot)), "load_angles")

    def step(self, n=1, sync=True):
        self._chk(self.L.tfg_step(self.h, n), "step")
        if sync:
            self.sync()

    def force_only(self, with_bonded=True):
        self._chk(self.L.tfg_force_only(self.h, 1 if with_bonded else 0), "force_only")
        self.sync()

    def pair_signature(self):
        """(count, hash) per particle id of the current binned state's pair set."""
        cnt = np.zeros(self.n, np.int32)
        hsh = np.zeros(self.n, np.uint32)
        self._chk(self.L.tfg_pair_signature(self.h, _ip(cnt), _up(hsh)), "pair_signature")
        return cnt, hsh

    def autotune(self):
        """Time the nonbonded pass's work splits on the current state; returns the chosen split."""
        v = C.c_int()
        self._chk(self.L.tfg_autotune(self.h, C.byref(v)), "autotune")
        return v.value

    def set_split(self, split):
        self._chk(self.L.tfg_set_split(self.h, split), "set_split")

    def tuning(self):
        """(split, warps per CTA, grab) the pair pass runs with (tfg_get_tuning)."""
        v = [C.c_int() for _ in range(3)]
        self._chk(self.L.tfg_get_tuning(self.h, *[C.byref(x) for x in v]), "get_tuning")
        return tuple(int(x.value) for x in v)

    def set_tuning(self, split, warps=8, grab=1):
        self._chk(self.L.tfg_set_tuning(self.h, split, warps, grab), "set_tuning")

    def set_stream(self, stream_ptr):
        """Order the engine's work on the caller's CUDA stream (cudaStream_t as int)."""
        self._chk(self.L.tfg_engine_set_stream(self.h, C.c_void_p(stream_ptr)), "set_stream")

    def sync(self):
        self._chk(self.L.tfg_sync(self.h), "sync")

    def idle(self):
        """True when the engine's stream has finished all queued work (does not block)."""
        v = C.c_int()
        self._chk(self.L.tfg_query(self.h, C.byref(v)), "query")
        return bool(v.value)

    def set_graphs(self, enable):
        self._chk(self.L.tfg_set_graphs(self.h, 1 if enable else 0), "set_graphs")

    def download(self):
        n, ns = self.n, self.nspec
        out = dict(x=np.zeros((n, 3), np.float32), xrel=np.zeros((n, 3), np.float32),
                   cell=np.zeros(n, np.int32), v=np.zeros((n, 3), np.float32), f=np.zeros((n, 3), np.float32),
                   density=np.zeros(n, np.float32), species=np.zeros((n, max(ns, 0)), np.float32),
                   q=np.zeros((n, max(ns, 0)), np.float32))
        self._chk(self.L.tfg_download(self.h, _fp(out["x"]), _fp(out["xrel"]), _ip(out["cell"]), _fp(out["v"]),
                                      _fp(out["f"]), _fp(out["density"]),
                                      _fp(out["species"]) if ns else None, _fp(out["q"]) if ns else None),
                  "download")
        return out

    def reductions(self):
        r = abi.Reductions()
        self._chk(self.L.tfg_get_reductions(self.h, C.byref(r)), "get_reductions")
        return r

    def set_pair_lists(self, enable):
        self._chk(self.L.tfg_set_pair_lists(self.h, 1 if enable else 0), "set_pair_lists")

    def pair_list(self):
        """(n_pairs, 2) int32 array of the interacting pairs (lower id, higher id), sorted,
        from the pair pass's own kernels (tfg_pair_list)."""
        n = C.c_int64()
        self._chk(self.L.tfg_pair_list(self.h, 0, None, C.byref(n)), "pair_list")
        out = np.zeros((max(int(n.value), 1), 2), np.int32)
        self._chk(self.L.tfg_pair_list(self.h, int(n.value), _ip(out), C.byref(n)), "pair_list")
        out = out[: int(n.value)]
        return out[np.lexsort((out[:, 1], out[:, 0]))]

    def set_deterministic(self, enable):
        """Pair pass without atomics: every run gives the same bits (tfg_set_deterministic)."""
        self._chk(self.L.tfg_set_deterministic(self.h, 1 if enable else 0), "set_deterministic")

    def resume(self, steps, q=None):
        """After load_binned: restore the engine time and the pending flux increments of a
        simulation saved mid-run (tfg_batch_resume on simulation 0)."""
        q = _conv(q, np.float32)
        self._chk(self.L.tfg_batch_resume(self.h, 0, int(steps), _fp(q)), "resume")

    def status(self):
        """0, or the first error (TFG_E_NAN / TFG_E_TOOFAST / TFG_E_RANGE) the simulation raised."""
        st = C.c_int()
        self._chk(self.L.tfg_batch_sim_status(self.h, 0, C.byref(st)), "batch_sim_status")
        return int(st.value)

    def verlet(self):
        """(rebuilds so far, largest displacement since the last rebuild) in Verlet mode."""
        nb, m = C.c_int64(), C.c_float()
        self._chk(self.L.tfg_get_verlet(self.h, C.byref(nb), C.byref(m)), "get_verlet")
        return int(nb.value), float(m.value)

    def set_phase_timing(self, enable):
        self._chk(self.L.tfg_set_phase_timing(self.h, 1 if enable else 0), "set_phase_timing")

    def phase_ms(self):
        ms = (C.c_float * 4)()
        self._chk(self.L.tfg_get_phase_ms(self.h, ms), "get_phase_ms")
        return list(ms)


class Batch(Engine):
    """Many independent simulations in one device arena (tfg_batch_*).  Engine-wide calls
    (step, sync, autotune, set_split, set_stream, phase_ms, set_bonded_potential) act on the
    whole batch; per-simulation calls go through the Sim handles add_sim returns."""

    def __init__(self, max_type, nr_species=0, device=0):
        self.L = lib()
        self.h = C.c_void_p()
        self.nspec = nr_species
        self.max_type = max_type
        rc = self.L.tfg_batch_create(device, max_type, nr_species, C.byref(self.h))
        if rc != 0:
            raise TfgError(rc, "tfg_batch_create")
        self.sims = {}
        self._keep = []

    def add_sim(self, desc):
        sid = C.c_int()
        self._chk(self.L.tfg_batch_add_sim(self.h, C.byref(desc), C.byref(sid)), "batch_add_sim")
        sim = Sim(self, sid.value, desc)
        self.sims[sid.value] = sim
        return sim

    def remove_sim(self, sim):
        sid = sim.sid if isinstance(sim, Sim) else int(sim)
        self._chk(self.L.tfg_batch_remove_sim(self.h, sid), "batch_remove_sim")
        self.sims.pop(sid, None)

    @property
    def n(self):
        """Particles of all loaded simulations (the length of pair_signature's arrays)."""
        return sum(s.n for s in self.sims.values())

    @n.setter
    def n(self, v):
        pass

    def live_count(self):
        v = C.c_int()
        self._chk(self.L.tfg_batch_sim_count(self.h, C.byref(v)), "batch_sim_count")
        return v.value

    def step(self, n=1, sync=True):
        self._chk(self.L.tfg_batch_step(self.h, n), "batch_step")
        if sync:
            self.sync()


class Sim:
    """One simulation of a Batch; method names match Engine's per-simulation calls."""

    def __init__(self, batch, sid, desc):
        self.b = batch
        self.L = batch.L
        self.sid = sid
        self.desc = desc
        self.nspec = desc.nr_species
        self.n = 0

    def _chk(self, rc, what):
        self.b._chk(rc, what)

    def set_type(self, t, dynamics, mass=1.0):
        self._chk(self.L.tfg_batch_set_type(self.b.h, self.sid, t, dynamics, mass), "batch_set_type")

    def set_potential(self, ti, tj, pot):
        ptr = pot.ptr if isinstance(pot, Potential) else pot
        self._chk(self.L.tfg_batch_set_potential(self.b.h, self.sid, ti, tj, ptr), "batch_set_potential")

    def add_flux(self, ti, tj, flux):
        self._chk(self.L.tfg_batch_add_flux(self.b.h, self.sid, ti, tj, C.byref(flux)), "batch_add_flux")

    def set_species_flags(self, flags):
        a = np.ascontiguousarray(flags, np.uint32)
        self._chk(self.L.tfg_batch_set_species_flags(self.b.h, self.sid, len(a), _up(a)), "batch_set_species_flags")

    def set_species_reset(self, values):
        a = np.ascontiguousarray(values, np.float32)
        self._chk(self.L.tfg_batch_set_species_reset(self.b.h, self.sid, len(a), _fp(a)), "batch_set_species_reset")

    def set_stop(self, step):
        """Stop this member at clock `step` (-1: run on) while the batch steps on."""
        self._chk(self.L.tfg_batch_set_stop(self.b.h, self.sid, int(step)), "batch_set_stop")

    def set_random_force(self, t, mean, std, duration_steps):
        self._chk(self.L.tfg_batch_set_random_force(self.b.h, self.sid, t, mean, std, duration_steps),
                  "batch_set_random_force")

    def set_bonded_potential(self, slot, pot):
        self.b.set_bonded_potential(slot, pot)

    def set_boundary(self, wall, kind, velocity=(0.0, 0.0, 0.0), restore=1.0, radius=0.0):
        b = abi.boundary(kind, velocity, restore, radius)
        self._chk(self.L.tfg_batch_set_boundary(self.b.h, self.sid, wall, C.byref(b)), "batch_set_boundary")

    def set_boundary_potential(self, wall, t, pot):
        ptr = pot.ptr if isinstance(pot, Potential) else pot
        self._chk(self.L.tfg_batch_set_boundary_potential(self.b.h, self.sid, wall, t, ptr),
                  "batch_set_boundary_potential")

    def load(self, x, v=None, type=None, radius=None, imass=None, flags=None, species=None, force_i=None):
        x = np.ascontiguousarray(x, np.float32)
        self.n = x.shape[0]
        v, radius, imass, species, force_i = (_conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = _conv(type, np.int32)
        flags = _conv(flags, np.uint32)
        self._chk(self.L.tfg_batch_load_particles(self.b.h, self.sid, self.n, _fp(x), _fp(v), _ip(type),
                                                  _fp(radius), _fp(imass), _up(flags), _fp(species),
                                                  _fp(force_i)), "batch_load_particles")

    def load_binned(self, cell, xrel, v=None, type=None, radius=None, imass=None, flags=None, species=None,
                    force_i=None):
        cell = np.ascontiguousarray(cell, np.int32)
        xrel = np.ascontiguousarray(xrel, np.float32)
        self.n = cell.shape[0]
        v, radius, imass, species, force_i = (_conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = _conv(type, np.int32)
        flags = _conv(flags, np.uint32)
        self._chk(self.L.tfg_batch_load_particles_binned(self.b.h, self.sid, self.n, _ip(cell), _fp(xrel), _fp(v),
                                                         _ip(type), _fp(radius), _fp(imass), _up(flags),
                                                         _fp(species), _fp(force_i)), "batch_load_particles_binned")

    def load_bonds(self, i, j, slot=None):
        i, j = (np.ascontiguousarray(a, np.int32) for a in (i, j))
        slot = _conv(slot, np.int32)
        self._chk(self.L.tfg_batch_load_bonds(self.b.h, self.sid, len(i), _ip(i), _ip(j), _ip(slot)),
                  "batch_load_bonds")

    def load_angles(self, i, j, k, slot=None):
        i, j, k = (np.ascontiguousarray(a, np.int32) for a in (i, j, k))
        slot = _conv(slot, np.int32)
        self._chk(self.L.tfg_batch_load_angles(self.b.h, self.sid, len(i), _ip(i), _ip(j), _ip(k), _ip(slot)),
                  "batch_load_angles")

    def download(self):
        n, ns = self.n, self.nspec
        out = dict(x=np.zeros((n, 3), np.float32), xrel=np.zeros((n, 3), np.float32),
                   cell=np.zeros(n, np.int32), v=np.zeros((n, 3), np.float32), f=np.zeros((n, 3), np.float32),
                   density=np.zeros(n, np.float32), species=np.zeros((n, max(ns, 0)), np.float32),
                   q=np.zeros((n, max(ns, 0)), np.float32))
        self._chk(self.L.tfg_batch_download(self.b.h, self.sid, _fp(out["x"]), _fp(out["xrel"]), _ip(out["cell"]),
                                            _fp(out["v"]), _fp(out["f"]), _fp(out["density"]),
                                            _fp(out["species"]) if ns else None, _fp(out["q"]) if ns else None),
                  "batch_download")
        return out

    def reductions(self):
        r = abi.Reductions()
        self._chk(self.L.tfg_batch_get_reductions(self.b.h, self.sid, C.byref(r)), "batch_get_reductions")
        return r

    def verlet(self):
        nb, m = C.c_int64(), C.c_float()
        self._chk(self.L.tfg_batch_get_verlet(self.b.h, self.sid, C.byref(nb), C.byref(m)), "batch_get_verlet")
        return int(nb.value), float(m.value)

    def resume(self, steps, q=None):
        """After load_binned: restore the engine time and pending flux increments."""
        q = _conv(q, np.float32)
        self._chk(self.L.tfg_batch_resume(self.b.h, self.sid, int(steps), _fp(q)), "batch_resume")

    def status(self):
        """0, or the first error (TFG_E_NAN / TFG_E_TOOFAST / TFG_E_RANGE) this simulation raised."""
        st = C.c_int()
        self._chk(self.L.tfg_batch_sim_status(self.b.h, self.sid, C.byref(st)), "batch_sim_status")
        return int(st.value)


def _potential(spec, cache, factory=None):
    make = factory or Potential.from_spec
    if cache is None:
        return make(spec)
    key = (getattr(make, "__qualname__", ""), spec.kind,
           tuple(sorted((k, tuple(v) if isinstance(v, list) else v) for k, v in spec.args.items())))
    p = cache.get(key)
    if p is None:
        p = cache[key] = make(spec)
    return p


def setup_model(eng, w, keep=None, pot_cache=None):
    """Apply a configs.Workload's interaction model and particles to an engine-like object
    (the GPU Engine, a batch Sim, or the CPU oracle share these method names).  Returns the
    Potential objects, which must stay alive while the engine uses their tables.  With a
    pot_cache dict, equal potential specifications share one table.  An engine-like object
    with a potential_from_spec method (the oracle) builds its own tables with it."""
    pots = []
    factory = getattr(eng, "potential_from_spec", None)
    for t in range(w.max_type):
        eng.set_type(t, w.dynamics[t], w.mass[t])
    for (ti, tj), spec in w.pots.items():
        p = _potential(spec, pot_cache, factory)
        pots.append(p)
        eng.set_potential(ti, tj, p.ptr)
    for (ti, tj, f) in w.fluxes:
        eng.add_flux(ti, tj, f)
    if w.random_force is not None:
        mean, std, dur = w.random_force
        for t in range(w.max_type):
            eng.set_random_force(t, mean, std, dur)
    for (t, mean, std, dur) in w.type_forces:
        eng.set_random_force(t, mean, std, dur)
    for (wall, kind, vel, restore, radius) in w.boundaries:
        eng.set_boundary(wall, kind, vel, restore, radius)
    if w.species_reset is not None:
        eng.set_species_reset(w.species_reset)
    for (wall, t, spec) in w.wall_pots:
        p = _potential(spec, pot_cache, factory)
        pots.append(p)
        eng.set_boundary_potential(wall, t, p.ptr)
    if w.bond_pot is not None:
        p = _potential(w.bond_pot, pot_cache, factory)
        pots.append(p)
        eng.set_bonded_potential(0, p.ptr)
    if w.angle_pot is not None:
        p = _potential(w.angle_pot, pot_cache, factory)
        pots.append(p)
        eng.set_bonded_potential(1, p.ptr)
    for slot, spec in enumerate(w.bonded_pots):
        p = _potential(spec, pot_cache, factory)
        pots.append(p)
        eng.set_bonded_potential(slot, p.ptr)
    eng.load(w.x, v=w.v, type=w.type, radius=w.radius, imass=w.imass, flags=w.flags_particles, species=w.species,
             force_i=w.force_i)
    if w.bonds is not None:
        bs = w.bond_slot if w.bond_slot is not None else np.zeros(len(w.bonds), np.int32)
        eng.load_bonds(w.bonds[:, 0], w.bonds[:, 1], bs)
    if w.angles is not None:
        aslot = w.angle_slot if w.angle_slot is not None else np.ones(len(w.angles), np.int32)
        eng.load_angles(w.angles[:, 0], w.angles[:, 1], w.angles[:, 2], aslot)
    if keep is not None:
        keep.extend(pots)
    return pots
