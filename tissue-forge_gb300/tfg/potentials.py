"""Potential factories mirroring TissueForge::Potential (tfPotential.cpp:2741-3142).

Tables are built by libtfg's host code exactly as potential_init builds them; the
returned object owns the table and exposes the C struct for the engine calls.
"""
import ctypes as C

from . import abi
from ._lib import lib


class Potential:
    def __init__(self, ptr, kind):
        self.ptr = ptr
        self.kind = kind

    def __del__(self):
        try:
            if self.ptr:
                lib().tfg_potential_free(self.ptr)
                self.ptr = None
        except Exception:
            pass

    @property
    def n(self):
        return self.ptr.contents.n

    def eval(self, r, ri=1.0, rj=1.0):
        """(energy, force/r) as potential_eval_ex computes them, or None out of range."""
        e = C.c_float()
        f = C.c_float()
        ok = lib().tfg_potential_eval(self.ptr, ri, rj, float(r) * float(r), C.byref(e), C.byref(f))
        return (e.value, f.value) if ok else None

    @staticmethod
    def _make(fn, *args, kind):
        p = abi.P_POT()
        rc = fn(*args, C.byref(p))
        if rc != 0:
            raise ValueError("%s failed: %s" % (kind, abi.STATUS_NAMES.get(rc, rc)))
        return Potential(p, kind)

    @classmethod
    def morse(cls, d=1.0, a=6.0, r0=0.0, min=0.0001, max=3.0, tol=0.001, shifted=True):
        return cls._make(lib().tfg_potential_morse, d, a, r0, min, max, tol, 1 if shifted else 0, kind="morse")

    @classmethod
    def lennard_jones_12_6(cls, min, max, A, B, tol=0.0):
        return cls._make(lib().tfg_potential_lennard_jones_12_6, min, max, A, B, tol, kind="lj")

    @classmethod
    def harmonic(cls, k, r0, min=-1.0, max=-1.0, tol=0.0):
        return cls._make(lib().tfg_potential_harmonic, k, r0, min, max, tol, kind="harmonic")

    @classmethod
    def harmonic_angle(cls, k, theta0, min=-1.0, max=-1.0, tol=0.0):
        return cls._make(lib().tfg_potential_harmonic_angle, k, theta0, min, max, tol, kind="harmonic_angle")

    @classmethod
    def dpd(cls, alpha=1.0, gamma=1.0, sigma=1.0, cutoff=1.0, shifted=False):
        return cls._make(lib().tfg_potential_dpd, alpha, gamma, sigma, cutoff, 1 if shifted else 0, kind="dpd")

    @classmethod
    def from_table(cls, kind, flags, alpha, r0_plusone, a, b, n, c, dpd=(0.0, 0.0, 0.0)):
        """A potential given as the reference stores it (struct Potential, tfPotential.h:213-253):
        the table is used as is, not rebuilt.  kind 1 is DPD (c unused)."""
        return RawPotential(kind, flags, alpha, r0_plusone, a, b, n, c, dpd)

    @classmethod
    def from_spec(cls, spec):
        a = spec.args
        if spec.kind == "table":
            return cls.from_table(a["kind"], a["flags"], a["alpha"], a["r0_plusone"], a["a"], a["b"], a["n"], a["c"],
                                  a.get("dpd", (0.0, 0.0, 0.0)))
        if spec.kind == "morse":
            return cls.morse(a["d"], a["a"], a["r0"], a["min"], a["max"], a["tol"], a["shifted"])
        if spec.kind == "lj":
            return cls.lennard_jones_12_6(a["min"], a["max"], a["A"], a["B"], a["tol"])
        if spec.kind == "harmonic":
            return cls.harmonic(a["k"], a["r0"], a["min"], a["max"], a["tol"])
        if spec.kind == "harmonic_angle":
            return cls.harmonic_angle(a["k"], a["theta0"], a["min"], a["max"], a["tol"])
        if spec.kind == "dpd":
            return cls.dpd(a["alpha"], a["gamma"], a["sigma"], a["cutoff"], a["shifted"])
        raise ValueError(spec.kind)


class RawPotential(Potential):
    """A potential whose descriptor and table live in Python memory (for tables read from a
    file).  set_potential copies both, so this object only needs to outlive that call."""

    def __init__(self, kind, flags, alpha, r0_plusone, a, b, n, c, dpd):
        import numpy as np
        self._c = np.ascontiguousarray(c, np.float32) if c is not None and len(c) else None
        st = abi.Potential()
        st.kind = int(kind)
        st.flags = int(flags)
        for k in range(4):
            st.alpha[k] = float(alpha[k]) if k < len(alpha) else 0.0
        st.r0_plusone = float(r0_plusone)
        st.a = float(a)
        st.b = float(b)
        st.n = int(n)
        st.c = self._c.ctypes.data_as(C.POINTER(C.c_float)) if self._c is not None else None
        st.dpd_alpha, st.dpd_gamma, st.dpd_sigma = (float(v) for v in dpd)
        self._st = st
        super().__init__(C.pointer(st), "table" if int(kind) != abi.POTENTIAL_KIND_DPD else "dpd")

    def __del__(self):
        self.ptr = None
