"""Boundary conditions on the CUDA path against the oracle: non-periodic axes (pair sets
bit-exact), FREESLIP and VELOCITY / NO_SLIP reflection, table and DPD wall potentials, alone
and inside a batch next to a periodic simulation."""
import numpy as np
import pytest

from helpers import FORCE_RTOL, force_error, make_gpu, make_oracle, small_dpd
from tfg import abi, configs
from tfg.configs import PotSpec
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu


def channel():
    """DPD slab between NO_SLIP walls in z with DPD wall potentials and a body force in x."""
    w = small_dpd()
    w.boundaries = [(4, abi.BOUNDARY_NO_SLIP, (0, 0, 0), 1.0, 0.0), (5, abi.BOUNDARY_NO_SLIP, (0, 0, 0), 1.0, 0.0)]
    w.wall_pots = [(-1, 0, PotSpec("dpd", dict(alpha=10.0, gamma=4.5, sigma=3.0, cutoff=1.0, shifted=False)))]
    return w


def sorting_box():
    """Cell sorting with FREESLIP x walls carrying a shifted Morse wall potential and moving
    VELOCITY y walls (restore 0.8); z periodic."""
    w = configs.cell_sorting(n=2500, side=15.0, seed=51)
    w.boundaries = [(0, abi.BOUNDARY_FREESLIP, (0, 0, 0), 1.0, 0.5), (1, abi.BOUNDARY_FREESLIP, (0, 0, 0), 1.0, 0.5),
                    (2, abi.BOUNDARY_VELOCITY, (0.5, 0, 0), 0.8, 0.0), (3, abi.BOUNDARY_VELOCITY, (-0.5, 0, 0), 0.8, 0.0)]
    morse = PotSpec("morse", dict(d=1.0, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True))
    w.wall_pots = [(0, 0, morse), (0, 1, morse), (1, 0, morse), (1, 1, morse)]
    return w


def _fext(w, fx=0.3):
    """force_i along x for every particle (a pressure gradient for the channel)."""
    return np.tile(np.array([[fx, 0.0, 0.0]], np.float32), (w.n, 1))


CASES = {"channel": channel, "sorting_box": sorting_box}


@pytest.mark.parametrize("name", sorted(CASES))
def test_boundary_pairs_and_forces(name):
    w = CASES[name]()
    g, o = make_gpu(w), make_oracle(w)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
    a, b = g.download(), o.download()
    assert force_error(a["f"], b["f"], o.fmag()) < FORCE_RTOL


@pytest.mark.parametrize("name", sorted(CASES))
def test_boundary_trajectory(name):
    w = CASES[name]()
    g, o = make_gpu(w), make_oracle(w)
    if name == "channel":
        fe = _fext(w)
        for e in (g, o):
            e.load(w.x, v=w.v, type=w.type, radius=w.radius, imass=w.imass, species=w.species, force_i=fe)
    g.step(8)
    o.step(8)
    a, b = g.download(), o.download()
    side = np.array(w.dim, np.float32)
    d = a["x"] - b["x"]
    d -= side * np.round(d / side)
    assert np.max(np.abs(d)) < 1e-3
    assert np.max(np.abs(a["v"] - b["v"])) < 1e-2
    # nothing left the box through a reflecting wall
    walls = [wall for (wall, kind, *_r) in w.boundaries if kind & (abi.BOUNDARY_FREESLIP | abi.BOUNDARY_VELOCITY |
                                                                    abi.BOUNDARY_NO_SLIP)]
    for wall in walls:
        ax = wall >> 1
        assert np.all(a["x"][:, ax] >= 0) and np.all(a["x"][:, ax] <= side[ax])


def test_boundaries_inside_a_batch():
    ws = [sorting_box(), configs.cell_sorting(n=900, side=12.5, seed=52)]
    b = Batch(2, 0)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.step(6)
    for w, s in zip(ws, sims):
        o = make_oracle(w)
        o.step(6)
        a, r = s.download(), o.download()
        side = np.array(w.dim, np.float32)
        d = a["x"] - r["x"]
        d -= side * np.round(d / side)
        assert np.max(np.abs(d)) < 1e-3


def test_resetting_boundary_matches_oracle():
    """BOUNDARY_RESETTING on the GPU: with no pair forces the integrator is bit-exact, so
    positions, cells and the species values (reset at the x crossings only) equal the
    oracle's bit for bit."""
    from test_cpu_boundary import resetting_box
    w = resetting_box()
    g, o = make_gpu(w), make_oracle(w)
    g.step(20)
    o.step(20)
    a, b = g.download(), o.download()
    assert np.array_equal(a["cell"], b["cell"])
    assert np.array_equal(a["xrel"].view(np.uint32), b["xrel"].view(np.uint32))
    assert np.array_equal(a["species"], b["species"])
    assert np.all(a["species"][:30, 0] == np.float32(0.25)) and np.all(a["species"][30:, 0] == 1.0)
