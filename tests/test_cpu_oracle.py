"""Known-answer tests of the CPU oracle (the checker of the GPU engine).

The reference's own tests hold no golden vectors for this path, so the oracle is pinned
here against closed-form results derived from the formulas it restates, and against
the published Philox4x32-10 known-answer vectors (Random123)."""
import math

import numpy as np
import pytest

import oracle as O
from helpers import force_error, make_oracle, small_bonded, small_cell_sorting, small_dpd
from tfg import Potential, abi, configs


def two_body(x0, x1, pot, side=20.0, cutoff=3.0, cells=6, dyn=abi.OVERDAMPED, species=None, flux=None,
             mode=O.MODE_NO_DENSITY, v=None):
    d = abi.engine_desc((0, 0, 0), (side,) * 3, (cells,) * 3, cutoff, 0.005, max_type=1,
                        nr_species=0 if species is None else species.shape[1])
    e = O.OracleEngine(d, mode)
    e.set_type(0, dyn)
    if pot is not None:
        e.set_potential(0, 0, pot.ptr)
    if flux is not None:
        e.add_flux(0, 0, flux)
    e.load(np.array([x0, x1], np.float32), v=v, species=species)
    return e


def test_philox_known_answers():
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("r", [0.9, 1.0, 1.3, 2.2])
def test_two_particle_morse_force(r):
    p = Potential.morse(d=3.0, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True)
    e = two_body([5.0, 5.0, 5.0], [5.0 + r, 5.0, 5.0], p)
    e.force_only()
    f = e.download()["f"]
    # Newton's third law holds exactly pair by pair
    assert np.array_equal(f[0], -f[1])
    ee, fr = p.eval(r)
    # part_i is the first particle: f_i = -fr * dx, dx = x_i - x_j = -r
    assert abs(f[0][0] - fr * r) <= 1e-6 * max(1.0, abs(fr * r))
    # against the analytic Morse derivative (table tolerance); below the table start
    # a = 1.01 the reference evaluates at a (tf_potential_eval.h:124)
    rr = max(r, 1.01)
    dU = 3.0 * (-10 * math.exp(-10 * (rr - 1)) + 10 * math.exp(-5 * (rr - 1)))
    assert abs(f[1][0] + dU) < 0.1 * max(1.0, abs(dU))


def test_two_particle_lj_across_periodic_boundary():
    p = Potential.lennard_jones_12_6(0.1, 2.5, 1.0, 1.0)
    # particles straddle the periodic boundary at x=0/20
    e = two_body([0.4, 5.0, 5.0], [19.2, 5.0, 5.0], p, cutoff=2.5, cells=8)
    e.record_pairs(True)
    e.force_only()
    assert len(e.pairs()) == 1
    f = e.download()["f"]
    r = 1.2
    ee, fr = p.eval(r)
    # particle 0 is pushed/pulled along +x relative to particle 1 at -0.8 (image)
    assert abs(abs(f[0][0]) - abs(fr * r)) < 1e-4 * abs(fr * r)
    assert np.allclose(f[0], -f[1])


def test_pairs_beyond_cutoff_excluded_inclusive_at_cutoff():
    p = Potential.lennard_jones_12_6(0.1, 2.5, 1.0, 1.0)
    e = two_body([5.0, 5.0, 5.0], [7.5, 5.0, 5.0], p, cutoff=2.5, cells=8)
    e.record_pairs(True)
    e.force_only()
    # r2 == cutoff^2 exactly is inside (tf_runner_dopair.cpp:172 uses r2 > cutoff2)
    assert len(e.pairs()) == 1
    e = two_body([5.0, 5.0, 5.0], [7.5001, 5.0, 5.0], p, cutoff=2.5, cells=8)
    e.record_pairs(True)
    e.force_only()
    assert len(e.pairs()) == 0


def test_fick_two_particle_exchange_conserves():
    f = abi.Flux()
    f.kind, f.type_a, f.type_b, f.index_a, f.index_b = abi.FLUX_FICK, 0, 0, 0, 0
    f.coef, f.decay, f.target, f.cutoff = 0.5, 0.0, 0.0, 1.0
    sp = np.array([[1.0], [0.0]], np.float32)
    e = two_body([5.0, 5.0, 5.0], [5.5, 5.0, 5.0], None, cutoff=1.0, cells=20, species=sp, flux=f,
                 dyn=abi.NEWTONIAN)
    e.step(1)
    s = e.download()["species"][:, 0]
    term = (1 - 0.5 / 1.0) ** 2
    q = term * 0.5 * (1.0 - 0.0)
    assert abs(s[0] - (1.0 - 0.005 * q)) < 1e-6
    assert abs(s[1] - 0.005 * q) < 1e-6
    assert abs(s.sum() - 1.0) < 1e-6


def test_dpd_reference_random_term_is_deterministic():
    pot = Potential.dpd(10.0, 4.5, 3.0, 1.0)
    v = np.array([[1.0, 0, 0], [-1.0, 0, 0]], np.float32)
    e = two_body([5.0, 5.0, 5.0], [5.6, 5.0, 5.0], pot, cutoff=1.0, cells=20, v=v,
                 mode=O.MODE_NO_DENSITY | O.MODE_REF_DPD_RANDOM)
    e.force_only()
    f = e.download()["f"]
    r = 0.6
    w = 1 - r / 1.0
    # e = dx/r = (-1,0,0); v_i - v_j = (2,0,0); e.v = -2
    F = 10.0 * w - 4.5 * w * w * (-2.0) + 3.0 * w / math.sqrt(0.005)
    assert abs(f[0][0] - (-F)) < 1e-4 * abs(F)
    assert np.allclose(f[0], -f[1])


def test_harmonic_bond_force():
    d = abi.engine_desc((0, 0, 0), (20.0,) * 3, (6,) * 3, 3.0, 0.005)
    e = O.OracleEngine(d, O.MODE_NO_DENSITY)
    hb = Potential.harmonic(100.0, 1.0)
    e.set_bonded_potential(0, hb.ptr)
    # bond across a cell boundary (x = 3.2 and 4.4 lie in cells 0 and 1)
    e.load(np.array([[3.2, 5.0, 5.0], [4.4, 5.0, 5.0]], np.float32))
    e.load_bonds([0], [1])
    e.force_only()
    f = e.download()["f"]
    # |F| = 2k(r - r0) = 40 within the table tolerance
    assert abs(f[0][0] - 40.0) < 0.5
    assert np.allclose(f[0], -f[1])


def test_harmonic_angle_force_restores_toward_theta0():
    d = abi.engine_desc((0, 0, 0), (20.0,) * 3, (6,) * 3, 3.0, 0.005)
    e = O.OracleEngine(d, O.MODE_NO_DENSITY)
    ha = Potential.harmonic_angle(20.0, math.pi)
    e.set_bonded_potential(1, ha.ptr)
    th = math.radians(120.0)
    x = np.array([[5.0 + math.cos(th), 5.0 + math.sin(th), 5.0], [5.0, 5.0, 5.0], [6.0, 5.0, 5.0]], np.float32)
    e.load(x)
    e.load_angles([0], [1], [2], [1])
    e.force_only()
    f = e.download()["f"]
    assert np.allclose(f.sum(axis=0), 0.0, atol=1e-4)
    # forces on the outer particles are perpendicular to their arms and open the angle
    rji = x[0] - x[1]
    rjk = x[2] - x[1]
    assert abs(np.dot(f[0], rji)) < 1e-4 and abs(np.dot(f[2], rjk)) < 1e-4
    assert f[2][1] < 0 and np.dot(f[0], [math.cos(th - math.pi / 2), math.sin(th - math.pi / 2), 0]) < 0


def test_setpartp_clamps_into_domain():
    d = abi.engine_desc((0, 0, 0), (20.0,) * 3, (6,) * 3, 3.0, 0.005)
    e = O.OracleEngine(d)
    cell, xrel = e.bin(np.array([[20.0, -1.0, 10.0], [0.0, 0.0, 0.0]], np.float32))
    assert cell[0] == (5 * 6 + 0) * 6 + 3
    assert np.all(xrel >= 0.0)


def test_overdamped_step_clamps_displacement_and_migrates():
    d = abi.engine_desc((0, 0, 0), (20.0,) * 3, (6,) * 3, 3.0, 0.005)
    e = O.OracleEngine(d, O.MODE_NO_DENSITY)
    e.set_type(0, abi.OVERDAMPED)
    h = 20.0 / 6
    x = np.array([[h - 0.01, 1.0, 1.0]], np.float32)
    fi = np.array([[1e6, 0.0, 0.0]], np.float32)    # huge force -> clamped to 0.05 h
    e.load(x, force_i=fi)
    e.step(1)
    out = e.download()
    assert out["cell"][0] == (1 * 6 + 0) * 6 + 0
    maxx = np.float32(np.float32(h) * np.float32(0.05))
    assert abs(out["x"][0][0] - (x[0][0] + maxx)) < 1e-5
    assert e.reductions().migrations == 1


@pytest.mark.parametrize("wl", ["cell_sorting", "bonded", "dpd"])
def test_sorted_window_matches_brute_force(wl):
    w = {"cell_sorting": configs.cell_sorting, "bonded": lambda: small_bonded(), "dpd": lambda: small_dpd()}[wl]()
    sets = []
    for mode in (0, O.MODE_BRUTE):
        e = make_oracle(w, mode)
        e.record_pairs(True)
        e.force_only()
        sets.append(e.pairs())
        assert e.stats()["window_skips"] == 0
    assert np.array_equal(sets[0], sets[1])


def test_threaded_oracle_matches_serial():
    w = small_bonded()
    a = make_oracle(w, 0, 1)
    b = make_oracle(w, 0, 4)
    a.force_only()
    b.force_only()
    fa, fb = a.download()["f"], b.download()["f"]
    assert force_error(fb, fa, a.fmag()) < 1e-5


def test_fp64_evaluation_close_to_fp32():
    w = small_cell_sorting()
    a = make_oracle(w, 0)
    b = make_oracle(w, O.MODE_FP64)
    a.force_only()
    b.force_only()
    f32 = a.download()["f"]
    f64 = b.forces_f64()[:, :3]
    assert force_error(f32, f64, a.fmag()) < 1e-5


def test_trajectory_is_deterministic():
    w = small_cell_sorting()
    a = make_oracle(w)
    b = make_oracle(w)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.download()["x"], b.download()["x"])
