"""Verlet mode of the oracle (engine_flag_verlet; engine_verlet_update, tfEngine.cpp:214-354):
the rebuild rule, particles kept in their cells between rebuilds, the Verlet integrator
branch, and no interacting pair lost while particles drift."""
import numpy as np
import pytest

import oracle as O
from tfg import abi, configs
from tfg.engine import setup_model


def _oracle(w, mode=0):
    e = O.OracleEngine(w.desc(), mode, 1)
    e._keep = setup_model(e, w)
    return e


def _dpd(skin=0.2):
    return configs.verlet(configs.dpd_droplets(n=3000, side=12.0, radius=4.0, seed=7), skin=skin)


def _min_image(d, side):
    return d - side * np.round(d / side)


def test_rebuild_rule_and_displacement():
    """Rebuild exactly when twice the largest displacement since the last rebuild exceeds the
    skin min(h) - cutoff; the displacement is measured from the positions at the rebuild."""
    w = _dpd()
    e = _oracle(w)
    side = w.dim[0]
    skin = min(d / c for d, c in zip(w.dim, w.cells)) - w.cutoff
    prev = e.download()["x"].astype(np.float64)   # positions entering step 1
    ref = None
    last_rebuilds = 0
    for step in range(1, 31):
        e.step(1)
        rebuilds, maxdx = e.verlet()
        if rebuilds > last_rebuilds:
            assert maxdx == 0.0
            ref = prev            # the rebuild re-bins the positions entering this step
        else:
            want = np.max(np.linalg.norm(_min_image(prev - ref, side), axis=1))
            assert abs(maxdx - want) < 1e-5
            assert 2.0 * maxdx <= skin
        if step > 1 and rebuilds > last_rebuilds:
            dx = np.max(np.linalg.norm(_min_image(prev - ref_before, side), axis=1))
            assert 2.0 * dx > skin - 1e-5
        ref_before = ref
        last_rebuilds = rebuilds
        prev = e.download()["x"].astype(np.float64)
    assert 5 <= last_rebuilds < 30


def test_particles_stay_in_their_cells_between_rebuilds():
    w = _dpd(skin=0.6)
    e = _oracle(w)
    h = np.array([d / c for d, c in zip(w.dim, w.cells)], np.float32)
    e.step(1)
    cell0 = e.download()["cell"].copy()
    outside = 0
    for _ in range(4):
        nb0 = e.verlet()[0]
        e.step(1)
        d = e.download()
        if e.verlet()[0] == nb0:
            assert np.array_equal(d["cell"], cell0)
            xr = d["xrel"]
            outside += int(np.sum(np.any((xr < 0) | (xr >= h), axis=1)))
        else:
            cell0 = d["cell"].copy()
    assert outside > 0     # some particles drifted out of their cells without moving


def test_no_pair_lost_while_drifting():
    """The pair set of every force pass is every pair within the cutoff (minimum image) at
    the positions entering the step, although particles have left their cells."""
    pytest.importorskip("scipy")
    from scipy.spatial import cKDTree
    w = _dpd(skin=0.4)
    e = _oracle(w)
    side, rc = w.dim[0], w.cutoff
    held = 0
    for _ in range(12):
        x = np.mod(e.download()["x"].astype(np.float64), side)
        nb0 = e.verlet()[0]
        e.record_pairs(True)
        e.step(1)
        got = {tuple(p) for p in e.pairs()}
        t = cKDTree(x, boxsize=side)
        inner = {tuple(p) for p in t.query_pairs(rc * (1 - 1e-4), output_type="ndarray")}
        outer = {tuple(p) for p in t.query_pairs(rc * (1 + 1e-4), output_type="ndarray")}
        assert inner <= got, "%d pairs within the cutoff were not evaluated" % len(inner - got)
        assert got <= outer
        held += e.verlet()[0] == nb0
    assert held >= 3


def test_verlet_integrator_branch():
    """Overdamped: v = f * imass, x += v * dt; Newtonian: v += f * dt * imass, x += v * dt;
    no velocity clamp (tf_engine_advance.cpp:367-427)."""
    lj = configs.PotSpec("lj", dict(min=0.1, max=1.0, A=1.0, B=1.0, tol=0.0))
    for dyn in (abi.OVERDAMPED, abi.NEWTONIAN):
        w = configs.Workload(name="two", origin=(0.0, 0.0, 0.0), dim=(8.0,) * 3, cells=(4, 4, 4), cutoff=1.0,
                             dt=0.01, steps=1, x=np.array([[3.1, 3.1, 3.1], [3.9, 3.1, 3.1]], np.float32),
                             type=np.zeros(2, np.int32), v=np.array([[50.0, 0, 0], [0, 0, 0]], np.float32),
                             dynamics=[dyn], flags=abi.ENGINE_VERLET)
        w.pots[(0, 0)] = lj
        e = _oracle(w)
        e.force_only()
        f = e.download()["f"].astype(np.float32)
        e = _oracle(w)
        e.step(1)
        d = e.download()
        dt = np.float32(0.01)
        v0 = w.v
        if dyn == abi.OVERDAMPED:
            v = f * np.float32(1.0)
        else:
            v = v0 + f * dt * np.float32(1.0)
        x = w.x + v * dt
        assert np.array_equal(d["v"], v)
        assert np.allclose(d["x"], x, atol=2e-6)
        # 50 * 0.01 = 0.5 > the reference's velocity clamp (0.05 * h / dt = 10): not applied
        if dyn == abi.NEWTONIAN:
            assert d["v"][0][0] > 40.0


def test_flux_increments_are_not_integrated():
    """The Verlet branch skips Fluxes_integrate: species values stay put with one flux step."""
    w = _dpd()
    e = _oracle(w)
    s0 = e.download()["species"].copy()
    e.step(3)
    assert np.array_equal(e.download()["species"], s0)
