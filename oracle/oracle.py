"""Python wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is the checker of the GPU engine.  Only the
tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  It
restates the reference's mdcore CPU engine; see tfg_oracle.cpp for the file:line
map.  It builds its own potential tables (tfo_potential.cpp, a restatement of
tfPotential.cpp's potential_init and factories) and never loads the product library.  Parity is unpinned by the reference (which cannot be built here and holds no
golden vectors for this path); it is pinned by known-answer tests and by the
fixtures under tests/golden/.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "tissue-forge_gb300"))
from tfg import abi  # noqa: E402  (struct layouts of include/tfg.h)

LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

MODE_FP64 = 1
MODE_BRUTE = 2
MODE_REF_DPD_RANDOM = 4
MODE_NO_DENSITY = 8


SOURCES = ("tfg_oracle.cpp", "tfo_potential.cpp")


def build(force=False):
    """Compile the oracle with the reference's FP rules (no FMA contraction)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(ROOT, "include", "tfg.h")]
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d)
                                                      for d in deps):
        return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I" + os.path.join(ROOT, "include"), "-o", LIB_PATH, *srcs, "-lpthread"]
    subprocess.check_call(cmd)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        E = C.c_void_p
        L.tfo_create.argtypes = [C.POINTER(abi.EngineDesc), C.c_int, C.c_int, C.POINTER(E)]
        L.tfo_destroy.argtypes = [E]
        L.tfo_destroy.restype = None
        L.tfo_set_type.argtypes = [E, C.c_int, C.c_int, C.c_float]
        L.tfo_set_potential.argtypes = [E, C.c_int, C.c_int, abi.P_POT]
        L.tfo_add_flux.argtypes = [E, C.c_int, C.c_int, C.POINTER(abi.Flux)]
        L.tfo_set_boundary.argtypes = [E, C.c_int, C.POINTER(abi.Boundary)]
        L.tfo_set_boundary_potential.argtypes = [E, C.c_int, C.c_int, abi.P_POT]
        L.tfo_set_species_flags.argtypes = [E, C.c_int, abi.U_P]
        L.tfo_set_species_reset.argtypes = [E, C.c_int, abi.F_P]
        L.tfo_set_random_force.argtypes = [E, C.c_int, C.c_float, C.c_float, C.c_int]
        L.tfo_load_particles.argtypes = [E, C.c_int, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P,
                                         abi.U_P, abi.F_P, abi.F_P]
        L.tfo_load_particles_binned.argtypes = [E, C.c_int, abi.I_P, abi.F_P, abi.F_P, abi.I_P, abi.F_P,
                                                abi.F_P, abi.U_P, abi.F_P, abi.F_P]
        L.tfo_bin.argtypes = [E, C.c_int, abi.F_P, abi.I_P, abi.F_P]
        L.tfo_set_bonded_potential.argtypes = [E, C.c_int, abi.P_POT]
        L.tfo_load_bonds.argtypes = [E, C.c_int, abi.I_P, abi.I_P, abi.I_P]
        L.tfo_load_angles.argtypes = [E, C.c_int, abi.I_P, abi.I_P, abi.I_P, abi.I_P]
        L.tfo_step.argtypes = [E, C.c_int]
        L.tfo_force_only.argtypes = [E, C.c_int]
        L.tfo_download.argtypes = [E, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P, abi.F_P, abi.F_P, abi.F_P]
        L.tfo_download_forces_f64.argtypes = [E, C.POINTER(C.c_double)]
        L.tfo_download_fmag.argtypes = [E, C.POINTER(C.c_double)]
        L.tfo_get_reductions.argtypes = [E, C.POINTER(abi.Reductions)]
        L.tfo_get_stats.argtypes = [E, C.POINTER(C.c_int64)]
        L.tfo_get_verlet.argtypes = [E, C.POINTER(C.c_int64), C.POINTER(C.c_float)]
        L.tfo_verlet_hold.argtypes = [E]
        L.tfo_signature.argtypes = [E, abi.I_P, abi.U_P]
        L.tfo_enable_signature.argtypes = [E, C.c_int]
        L.tfo_record_pairs.argtypes = [E, C.c_int]
        L.tfo_get_pairs.argtypes = [E, abi.I_P, C.c_int64]
        L.tfo_get_pairs.restype = C.c_int64
        L.tfo_philox_probe.argtypes = [C.c_uint32] * 6 + [C.POINTER(C.c_uint32)]
        L.tfo_philox_probe.restype = C.c_uint32
        PP = C.POINTER(abi.P_POT)
        f = C.c_float
        L.tfo_potential_morse.argtypes = [f, f, f, f, f, f, C.c_int, PP]
        L.tfo_potential_lennard_jones_12_6.argtypes = [f, f, f, f, f, PP]
        L.tfo_potential_harmonic.argtypes = [f, f, f, f, f, PP]
        L.tfo_potential_harmonic_angle.argtypes = [f, f, f, f, f, PP]
        L.tfo_potential_dpd.argtypes = [f, f, f, f, C.c_int, PP]
        L.tfo_potential_free.argtypes = [abi.P_POT]
        L.tfo_potential_free.restype = None
    return _lib


def _fp(a):
    return None if a is None else a.ctypes.data_as(abi.F_P)


def _ip(a):
    return None if a is None else a.ctypes.data_as(abi.I_P)


def _up(a):
    return None if a is None else a.ctypes.data_as(abi.U_P)


def _chk(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed: %s" % (what, abi.STATUS_NAMES.get(rc, rc)))


class OraclePotential:
    """A potential table built by the oracle's own restatement of the reference's
    potential_init and factories (tfo_potential.cpp), never by the product library."""

    def __init__(self, ptr, kind):
        self.ptr = ptr
        self.kind = kind

    def __del__(self):
        try:
            if self.ptr:
                lib().tfo_potential_free(self.ptr)
                self.ptr = None
        except Exception:
            pass

    @property
    def n(self):
        return self.ptr.contents.n

    def table(self):
        """(kind, flags, alpha[4], r0_plusone, a, b, n, c as float32 array or None)."""
        p = self.ptr.contents
        c = None
        if p.c:
            c = np.ctypeslib.as_array(p.c, shape=((p.n + 1) * 8,)).copy()
        return (p.kind, p.flags, tuple(p.alpha), p.r0_plusone, p.a, p.b, p.n, c)

    @classmethod
    def _make(cls, fn, *args, kind):
        p = abi.P_POT()
        rc = fn(*args, C.byref(p))
        if rc != 0:
            raise ValueError("oracle %s failed: %s" % (kind, abi.STATUS_NAMES.get(rc, rc)))
        return cls(p, kind)

    @classmethod
    def from_spec(cls, spec):
        """Build the potential a configs.PotSpec names (factory arguments, or a stored table)."""
        a = spec.args
        L = lib()
        if spec.kind == "table":
            from tfg.potentials import RawPotential   # holds a given table; builds nothing
            return RawPotential(a["kind"], a["flags"], a["alpha"], a["r0_plusone"], a["a"], a["b"], a["n"],
                                a["c"], a.get("dpd", (0.0, 0.0, 0.0)))
        if spec.kind == "morse":
            return cls._make(L.tfo_potential_morse, a["d"], a["a"], a["r0"], a["min"], a["max"], a["tol"],
                             1 if a["shifted"] else 0, kind="morse")
        if spec.kind == "lj":
            return cls._make(L.tfo_potential_lennard_jones_12_6, a["min"], a["max"], a["A"], a["B"], a["tol"],
                             kind="lj")
        if spec.kind == "harmonic":
            return cls._make(L.tfo_potential_harmonic, a["k"], a["r0"], a["min"], a["max"], a["tol"],
                             kind="harmonic")
        if spec.kind == "harmonic_angle":
            return cls._make(L.tfo_potential_harmonic_angle, a["k"], a["theta0"], a["min"], a["max"], a["tol"],
                             kind="harmonic_angle")
        if spec.kind == "dpd":
            return cls._make(L.tfo_potential_dpd, a["alpha"], a["gamma"], a["sigma"], a["cutoff"],
                             1 if a["shifted"] else 0, kind="dpd")
        raise ValueError(spec.kind)


class OracleEngine:
    """CPU restatement of one Tissue Forge engine (space + potentials + fluxes + bonds)."""

    def __init__(self, desc, mode=0, threads=1, signature=True):
        self.L = lib()
        self.h = C.c_void_p()
        self.desc = desc
        self.nspec = desc.nr_species
        _chk(self.L.tfo_create(C.byref(desc), mode, threads, C.byref(self.h)), "create")
        _chk(self.L.tfo_enable_signature(self.h, 1 if signature else 0), "enable_signature")
        self.n = 0

    def close(self):
        if self.h:
            self.L.tfo_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_type(self, t, dynamics, mass=1.0):
        _chk(self.L.tfo_set_type(self.h, t, dynamics, mass), "set_type")

    @staticmethod
    def potential_from_spec(spec):
        """The oracle builds its own tables (setup_model calls this when present)."""
        return OraclePotential.from_spec(spec)

    def set_potential(self, ti, tj, pot):
        _chk(self.L.tfo_set_potential(self.h, ti, tj, pot), "set_potential")

    def add_flux(self, ti, tj, flux):
        _chk(self.L.tfo_add_flux(self.h, ti, tj, C.byref(flux)), "add_flux")

    def set_boundary(self, wall, kind, velocity=(0.0, 0.0, 0.0), restore=1.0, radius=0.0):
        b = abi.boundary(kind, velocity, restore, radius)
        _chk(self.L.tfo_set_boundary(self.h, wall, C.byref(b)), "set_boundary")

    def set_boundary_potential(self, wall, t, pot):
        _chk(self.L.tfo_set_boundary_potential(self.h, wall, t, pot), "set_boundary_potential")

    def set_species_flags(self, flags):
        a = np.ascontiguousarray(flags, np.uint32)
        _chk(self.L.tfo_set_species_flags(self.h, len(a), _up(a)), "set_species_flags")

    def set_random_force(self, t, mean, std, duration_steps):
        _chk(self.L.tfo_set_random_force(self.h, t, mean, std, duration_steps), "set_random_force")

    def set_species_reset(self, values):
        a = np.ascontiguousarray(values, np.float32)
        _chk(self.L.tfo_set_species_reset(self.h, len(a), _fp(a)), "set_species_reset")

    def set_bonded_potential(self, slot, pot):
        _chk(self.L.tfo_set_bonded_potential(self.h, slot, pot), "set_bonded_potential")

    def load(self, x, v=None, type=None, radius=None, imass=None, flags=None, species=None, force_i=None):
        x = np.ascontiguousarray(x, np.float32)
        self.n = x.shape[0]
        conv = lambda a, dt: None if a is None else np.ascontiguousarray(a, dt)
        v, radius, imass, species, force_i = (conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = conv(type, np.int32)
        flags = conv(flags, np.uint32)
        _chk(self.L.tfo_load_particles(self.h, self.n, _fp(x), _fp(v), _ip(type), _fp(radius), _fp(imass),
                                       _up(flags), _fp(species), _fp(force_i)), "load")

    def load_binned(self, cell, xrel, v=None, type=None, radius=None, imass=None, flags=None, species=None,
                    force_i=None):
        cell = np.ascontiguousarray(cell, np.int32)
        xrel = np.ascontiguousarray(xrel, np.float32)
        self.n = cell.shape[0]
        conv = lambda a, dt: None if a is None else np.ascontiguousarray(a, dt)
        v, radius, imass, species, force_i = (conv(a, np.float32) for a in (v, radius, imass, species, force_i))
        type = conv(type, np.int32)
        flags = conv(flags, np.uint32)
        _chk(self.L.tfo_load_particles_binned(self.h, self.n, _ip(cell), _fp(xrel), _fp(v), _ip(type),
                                              _fp(radius), _fp(imass), _up(flags), _fp(species), _fp(force_i)),
             "load_binned")

    def bin(self, x):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        cell = np.zeros(n, np.int32)
        xrel = np.zeros((n, 3), np.float32)
        _chk(self.L.tfo_bin(self.h, n, _fp(x), _ip(cell), _fp(xrel)), "bin")
        return cell, xrel

    def load_bonds(self, i, j, slot=None):
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        slot = None if slot is None else np.ascontiguousarray(slot, np.int32)
        _chk(self.L.tfo_load_bonds(self.h, len(i), _ip(i), _ip(j), _ip(slot)), "load_bonds")

    def load_angles(self, i, j, k, slot=None):
        i, j, k = (np.ascontiguousarray(a, np.int32) for a in (i, j, k))
        slot = None if slot is None else np.ascontiguousarray(slot, np.int32)
        _chk(self.L.tfo_load_angles(self.h, len(i), _ip(i), _ip(j), _ip(k), _ip(slot)), "load_angles")

    def step(self, n=1):
        _chk(self.L.tfo_step(self.h, n), "step")

    def force_only(self, with_bonded=True):
        _chk(self.L.tfo_force_only(self.h, 1 if with_bonded else 0), "force_only")

    def download(self):
        n, ns = self.n, self.nspec
        out = dict(x=np.zeros((n, 3), np.float32), xrel=np.zeros((n, 3), np.float32),
                   cell=np.zeros(n, np.int32), v=np.zeros((n, 3), np.float32), f=np.zeros((n, 3), np.float32),
                   density=np.zeros(n, np.float32), species=np.zeros((n, max(ns, 0)), np.float32),
                   q=np.zeros((n, max(ns, 0)), np.float32))
        _chk(self.L.tfo_download(self.h, _fp(out["x"]), _fp(out["xrel"]), _ip(out["cell"]), _fp(out["v"]),
                                 _fp(out["f"]), _fp(out["density"]),
                                 _fp(out["species"]) if ns else None, _fp(out["q"]) if ns else None), "download")
        return out

    def forces_f64(self):
        f = np.zeros((self.n, 4), np.float64)
        _chk(self.L.tfo_download_forces_f64(self.h, f.ctypes.data_as(C.POINTER(C.c_double))), "forces_f64")
        return f

    def fmag(self):
        m = np.zeros(self.n, np.float64)
        _chk(self.L.tfo_download_fmag(self.h, m.ctypes.data_as(C.POINTER(C.c_double))), "fmag")
        return m

    def signature(self):
        """(count, hash) per particle id of the last force pass, accumulated in the pair loop."""
        cnt = np.zeros(self.n, np.int32)
        hsh = np.zeros(self.n, np.uint32)
        _chk(self.L.tfo_signature(self.h, _ip(cnt), _up(hsh)), "signature")
        return cnt, hsh

    def pair_signature(self):
        """(count, hash) per particle id from the recorded pair list (same mix as the GPU)."""
        pr = self.pairs()
        cnt = np.zeros(self.n, np.int64)
        hsh = np.zeros(self.n, np.uint64)
        if len(pr):
            a, b = pr[:, 0].astype(np.int64), pr[:, 1].astype(np.int64)
            np.add.at(cnt, a, 1)
            np.add.at(cnt, b, 1)
            np.add.at(hsh, a, sig_mix(b))
            np.add.at(hsh, b, sig_mix(a))
        return cnt.astype(np.int32), (hsh & 0xFFFFFFFF).astype(np.uint32)

    def reductions(self):
        r = abi.Reductions()
        _chk(self.L.tfo_get_reductions(self.h, C.byref(r)), "reductions")
        return r

    def verlet(self):
        """(rebuilds so far, space::maxdx after the last step) in Verlet mode."""
        nb, m = C.c_int64(), C.c_float()
        _chk(self.L.tfo_get_verlet(self.h, C.byref(nb), C.byref(m)), "verlet")
        return int(nb.value), float(m.value)

    def verlet_hold(self):
        """Take the current cells and positions as the last Verlet rebuild's."""
        _chk(self.L.tfo_verlet_hold(self.h), "verlet_hold")

    def stats(self):
        s = (C.c_int64 * 3)()
        _chk(self.L.tfo_get_stats(self.h, s), "stats")
        return dict(window_skips=s[0], straight_angles=s[1], tasks=s[2])

    def record_pairs(self, on=True):
        _chk(self.L.tfo_record_pairs(self.h, 1 if on else 0), "record_pairs")

    def pairs(self):
        n = self.L.tfo_get_pairs(self.h, None, 0)
        out = np.zeros((n, 2), np.int32)
        self.L.tfo_get_pairs(self.h, _ip(out), n)
        return out


def sig_mix(ids):
    """32-bit mix of particle ids used by the pair signature (uint64 arrays in, out)."""
    x = (ids.astype(np.uint64) * np.uint64(2654435761) + np.uint64(0x9E3779B9)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x85EBCA6B)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(13)
    return x


def philox(c, k):
    out = (C.c_uint32 * 4)()
    lib().tfo_philox_probe(c[0], c[1], c[2], c[3], k[0], k[1], out)
    return list(out)
