"""The product's potential tables against the oracle's own table builder.

The oracle restates potential_init and the Morse, Lennard-Jones 12-6, harmonic,
harmonic-angle and DPD factories from source/mdcore/src/tfPotential.cpp:131-134,
192-245, 343-401, 550-626, 1057-1109, 1396-2040, 2188-2283, 2741-2751, 2961-3003,
3068-3084, 3128-3142 and tfDPDPotential.cpp:32-43 in oracle/tfo_potential.cpp, written
independently of libtfg.  Every potential the workloads and tests use, and a seeded
sweep of factory arguments, must come out of both builders word for word: kind, flags,
the index transform alpha[0..3], r0_plusone, a, b, the interval count n and every
coefficient c[0 .. 8(n+1)).
"""
import math

import numpy as np
import pytest

import oracle as O
from tfg import configs
from tfg.potentials import Potential


def _product_table(spec):
    p = Potential.from_spec(spec)
    st = p.ptr.contents
    c = None
    if st.c:
        c = np.ctypeslib.as_array(st.c, shape=((st.n + 1) * 8,)).copy()
    return p, (st.kind, st.flags, tuple(st.alpha), st.r0_plusone, st.a, st.b, st.n, c)


def _bits(v):
    return np.float32(v).view(np.uint32)


def _assert_same(spec, may_refuse=False):
    try:
        op = O.OraclePotential.from_spec(spec)
    except ValueError:
        # the reference refuses tables that need more than potential_ivalsmax intervals
        assert may_refuse, spec
        with pytest.raises(ValueError):
            _product_table(spec)
        return None
    o = op.table()
    keep, p = _product_table(spec)
    kind, flags, alpha, r0p, a, b, n, c = o
    assert (kind, flags, n) == p[0:2] + (p[6],), (spec, o[:7], p[:7])
    for name, x, y in (("alpha", alpha, p[2]), ("r0_plusone", (r0p,), (p[3],)), ("a", (a,), (p[4],)),
                       ("b", (b,), (p[5],))):
        assert [_bits(v) for v in x] == [_bits(v) for v in y], (name, spec, x, y)
    if c is None:
        assert p[7] is None
    else:
        assert p[7] is not None and len(c) == len(p[7]) == 8 * (n + 1)
        diff = np.nonzero(c.view(np.uint32) != p[7].view(np.uint32))[0]
        assert len(diff) == 0, (spec, "table words differ at", diff[:10])
    return o


def _workload_specs():
    specs = []
    specs += list(configs.cell_sorting().pots.values())
    specs += list(configs.dpd_droplets(n=2000, side=16.0, radius=4.0).pots.values())
    w = configs.bonded_fluid(n=16 * 200)
    specs += list(w.pots.values()) + [w.bond_pot, w.angle_pot]
    specs += list(configs.lj_fluid(n=4000).pots.values())
    for w in configs.ensemble():
        specs += list(w.pots.values())
    for req in configs.served_requests(count=40):
        specs += list(configs.request_workload(req).pots.values())
    return specs


def _test_specs():
    P = configs.PotSpec
    return [
        P("lj", dict(min=0.1, max=1.0, A=1.0, B=1.0, tol=0.0)),
        P("lj", dict(min=0.1, max=2.0, A=1.0, B=1.0, tol=0.0)),
        P("lj", dict(min=0.1, max=1.0, A=0.01, B=0.02, tol=0.0)),
        P("morse", dict(d=1.0, a=3.0, r0=1.0, min=0.2, max=3.0, tol=0.01, shifted=True)),
        P("morse", dict(d=1.0, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True)),
        P("morse", dict(d=1.25, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True)),
        P("morse", dict(d=1.0, a=6.0, r0=0.0, min=0.0001, max=3.0, tol=0.001, shifted=True)),
        P("harmonic", dict(k=100.0, r0=1.0, min=-1.0, max=-1.0, tol=0.0)),
        P("harmonic_angle", dict(k=20.0, theta0=math.pi, min=-1.0, max=-1.0, tol=0.0)),
        P("dpd", dict(alpha=10.0, gamma=4.5, sigma=3.0, cutoff=1.0, shifted=False)),
        P("dpd", dict(alpha=25.0, gamma=3.0, sigma=1.0, cutoff=1.0, shifted=True)),
    ]


def _unique(specs):
    seen, out = set(), []
    for s in specs:
        key = (s.kind, tuple(sorted(s.args.items())))
        if key not in seen:
            seen.add(key)
            out.append(s)
    return out


def test_tables_of_every_workload_potential_match_the_oracle():
    specs = _unique(_workload_specs())
    kinds = {s.kind for s in specs}
    assert {"morse", "dpd", "lj", "harmonic", "harmonic_angle"} <= kinds
    for s in specs:
        _assert_same(s)


@pytest.mark.parametrize("spec", _test_specs(), ids=lambda s: s.kind)
def test_tables_of_test_potentials_match_the_oracle(spec):
    _assert_same(spec)


def test_tables_match_the_oracle_over_a_parameter_sweep():
    """A seeded sweep of factory arguments, both Morse forms, LJ, harmonic and angles."""
    rng = np.random.default_rng(20240611)
    P = configs.PotSpec
    n_tables = 0
    for it in range(150):
        k = it % 5
        u = lambda lo, hi: float(rng.uniform(lo, hi))
        if k == 0:
            s = P("morse", dict(d=u(0.1, 5), a=u(1, 8), r0=u(0.5, 2), min=u(0.005, 0.5), max=u(2, 5),
                                tol=float(rng.choice([0.001, 0.01, 0.0005])), shifted=True))
        elif k == 1:
            s = P("morse", dict(d=u(0.1, 5), a=u(1, 8), r0=u(0.5, 2), min=u(0.2, 0.6), max=u(2, 5),
                                tol=float(rng.choice([0.001, 0.01])), shifted=False))
        elif k == 2:
            s = P("lj", dict(min=u(0.05, 0.8), max=u(1.2, 4), A=u(0.1, 3), B=u(0.1, 3), tol=0.0))
        elif k == 3:
            s = P("harmonic", dict(k=u(1, 200), r0=u(0.3, 3), min=-1.0, max=-1.0, tol=0.0))
        else:
            s = P("harmonic_angle", dict(k=u(1, 50), theta0=u(0.5, 3.14), min=-1.0, max=-1.0, tol=0.0))
        o = _assert_same(s, may_refuse=True)
        if o is not None:
            n_tables += 1
    assert n_tables > 120


def test_oracle_builder_refuses_what_the_product_refuses():
    P = configs.PotSpec
    for s in (P("lj", dict(min=2.5, max=0.1, A=1.0, B=1.0, tol=0.0)),
              P("morse", dict(d=1.0, a=6.0, r0=0.0, min=1.0, max=0.0, tol=0.001, shifted=True))):
        with pytest.raises(ValueError):
            O.OraclePotential.from_spec(s)
        with pytest.raises(ValueError):
            Potential.from_spec(s)
