"""Table construction (potential_init, tfPotential.cpp:1396-1634) against the analytic
functions the reference tabulates.  The bisection guarantees the energy error per
interval (relative to max(|f|,1)) is below the requested tolerance."""
import math

import numpy as np
import pytest

from tfg import Potential, abi


def morse_shifted(r, d, a):
    return d * (math.exp(-2 * a * (r - 1)) - 2 * math.exp(-a * (r - 1)))


@pytest.mark.parametrize("d", [3.0, 0.5, 1.25])
def test_morse_table_within_tolerance(d):
    p = Potential.morse(d=d, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True)
    st = p.ptr.contents
    assert st.flags & abi.POTENTIAL_SHIFTED
    assert abs(st.r0_plusone - 2.0) < 1e-7
    assert 1 <= st.n <= 3048
    # domain shifted by +1 (tfPotential.cpp:2271)
    assert abs(st.a - 1.01) < 1e-6 and abs(st.b - 4.0) < 1e-6
    worst = 0.0
    for r in np.linspace(1.012, 2.999, 3000):
        e, f = p.eval(r)       # radii 1+1, r0_plusone 2 -> r' = r
        ref = morse_shifted(r, d, 5.0)
        worst = max(worst, abs(e - ref) / max(1.0, abs(ref)))
    assert worst < 0.001 * 1.05


def test_lj_table_within_tolerance():
    p = Potential.lennard_jones_12_6(0.1, 2.5, 1.0, 1.0)
    st = p.ptr.contents
    assert st.n <= 3048
    worst = 0.0
    for r in np.linspace(0.11, 2.49, 4000):
        e, f = p.eval(r)
        ref = r ** -12 - r ** -6
        worst = max(worst, abs(e - ref) / max(1.0, abs(ref)))
    assert worst < 0.0024 * 1.05


def test_harmonic_table_and_flags():
    p = Potential.harmonic(100.0, 1.0)
    st = p.ptr.contents
    # potential_create_harmonic: flags = POTENTIAL_HARMONIC & POTENTIAL_R2 == 0 (tfPotential.cpp:374)
    assert st.flags == 0
    assert st.a == 0.0 and abs(st.b - 2.0) < 1e-6
    # interval 0 is the linear continuation with c[1] = 1/a = inf (a == 0)
    assert math.isinf(st.c[1])
    for r in np.linspace(0.5, 1.9, 50):
        e, f = p.eval(r)
        assert abs(e - 100.0 * (r - 1.0) ** 2) < 0.02 * 2.0 * 1.05
        assert abs(f * r - 200.0 * (r - 1.0)) < 0.05 * 200


def test_harmonic_angle_table():
    p = Potential.harmonic_angle(20.0, math.pi)
    st = p.ptr.contents
    assert st.flags == (abi.POTENTIAL_ANGLE | abi.POTENTIAL_HARMONIC)
    assert abs(st.a + 1.0) < 1e-5 and abs(st.b - 1.0) < 1e-5
    assert st.n >= 1


def test_dpd_fields():
    p = Potential.dpd(10.0, 4.5, 3.0, 1.0)
    st = p.ptr.contents
    assert st.kind == abi.POTENTIAL_KIND_DPD
    assert abs(st.a - math.sqrt(np.finfo(np.float32).eps)) < 1e-7
    assert st.b == 1.0 and st.dpd_alpha == 10.0 and st.dpd_gamma == 4.5 and st.dpd_sigma == 3.0


def test_bad_arguments_rejected():
    with pytest.raises(ValueError):
        Potential.lennard_jones_12_6(2.5, 0.1, 1.0, 1.0)
    with pytest.raises(ValueError):
        Potential.morse(max=0.0, min=1.0)
