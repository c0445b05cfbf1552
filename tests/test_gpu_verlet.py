"""Verlet mode on the GPU (TFG_ENGINE_VERLET) against the oracle's Verlet mode: rebuild
decisions, the pair set with particles outside their cells (bit-exact), trajectories, and
batches that mix Verlet and cell-list simulations."""
import dataclasses

import numpy as np
import pytest

import oracle as O
from helpers import make_gpu, make_oracle, small_bonded, small_dpd
from tfg import abi, configs
from tfg.engine import Batch, Engine, setup_model

pytestmark = pytest.mark.gpu


def _relaxed(w, steps=200):
    """`w` with its positions after `steps` overdamped cell-list steps under the reference's
    displacement clamp.  The Verlet integrator has no clamp, so overlapping chain beads of
    the generated start would fly apart."""
    base = dataclasses.replace(w, flags=w.flags & ~abi.ENGINE_VERLET, dynamics=[abi.OVERDAMPED] * w.max_type)
    o = make_oracle(base)
    o.step(steps)
    return dataclasses.replace(w, x=configs.in_box(o.download()["x"], w.dim[0]))


WORKLOADS = {
    # 4,000 particles, 5^3 cells of edge 4 (skin 1)
    "cell_sorting": lambda: configs.verlet(configs.cell_sorting(random_force=(0.0, 2.0, 1)), skin=0.3),
    # 4,000 DPD particles with flux, 8^3 cells of edge 1.5 (skin 0.5)
    "dpd": lambda: configs.verlet(small_dpd(), skin=0.4),
    # 8,000 LJ particles in chains, relaxed first (200 steps); skin 0.75
    "bonded": lambda: _relaxed(configs.verlet(small_bonded(), skin=0.3)),
}


@pytest.fixture(params=sorted(WORKLOADS))
def wl(request):
    return request.param, WORKLOADS[request.param]()


def _dev(a, b, dim):
    side = np.array(dim, np.float32)
    d = a - b
    d -= side * np.round(d / side)
    return np.abs(d).max(axis=1)


def test_trajectory_and_rebuilds_match_oracle(wl):
    name, w = wl
    g = make_gpu(w)
    o = make_oracle(w)
    for _ in range(12):
        g.step(1)
        o.step(1)
        assert g.verlet()[0] == o.verlet()[0], name
    a, b = g.download(), o.download()
    # same bar as the cell-list trajectories: summation order differs from the oracle's
    dev = _dev(a["x"], b["x"], w.dim)
    assert dev.max() < 2e-3, "max position deviation %.3g" % dev.max()
    assert np.percentile(dev, 99) < 1e-4
    assert np.array_equal(a["cell"], b["cell"])
    if w.nr_species:
        assert np.max(np.abs(a["species"] - b["species"])) < 1e-4
    rb, maxdx = g.verlet()
    assert abs(maxdx - o.verlet()[1]) < 1e-4


def test_pair_set_with_particles_outside_their_cells_bitexact(wl):
    name, w = wl
    o = make_oracle(w)
    o.step(8)
    d = o.download()
    h = np.array([dm / c for dm, c in zip(w.dim, w.cells)], np.float32)
    assert np.any((d["xrel"] < 0) | (d["xrel"] >= h)), "no particle outside its cell"
    args = dict(v=d["v"], type=w.type, radius=w.radius, imass=w.imass,
                species=d["species"] if w.nr_species else None)
    g = make_gpu(w)
    g.load_binned(d["cell"], d["xrel"], **args)
    gc, gh = g.pair_signature()
    r = O.OracleEngine(w.desc(), O.MODE_BRUTE, 1)
    r._keep = setup_model(r, w)
    r.load_binned(d["cell"], d["xrel"], **args)
    r.verlet_hold()
    r.force_only()
    rc, rh = r.signature()
    assert np.array_equal(gc, rc), "pair counts differ for %d particles" % int((gc != rc).sum())
    assert np.array_equal(gh, rh)


def test_batch_mixing_verlet_and_cell_list_members_equals_alone():
    ws = [configs.verlet(configs.cell_sorting(n=2500, side=17.0, seed=21, random_force=(0.0, 2.0, 1)), skin=0.3),
          configs.cell_sorting(n=900, side=12.5, depth_ab=1.7, seed=22),
          configs.verlet(configs.cell_sorting(n=6000, side=22.9, seed=23, random_force=(0.0, 2.0, 1)), skin=0.5)]
    b = Batch(ws[0].max_type, ws[0].nr_species)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.step(10)
    for w, s in zip(ws, sims):
        g = make_gpu(w)
        g.step(10)
        a, r = s.download(), g.download()
        assert np.array_equal(a["cell"], r["cell"]), w.name
        assert _dev(a["x"], r["x"], w.dim).max() < 1e-3, w.name
        if w.flags:
            assert s.verlet()[0] == g.verlet()[0] > 1, w.name


def _held_signature(w, d):
    """Oracle pair signature (brute force) of a binned state taken as the last rebuild's."""
    r = O.OracleEngine(w.desc(), O.MODE_BRUTE, 1)
    r._keep = setup_model(r, w)
    r.load_binned(d["cell"], d["xrel"], v=d["v"], type=w.type, radius=w.radius, imass=w.imass,
                  species=d["species"] if w.nr_species else None)
    r.verlet_hold()
    r.force_only()
    return r.signature()


def _walk_and_compare(g, w, steps, on_step=None):
    """Step `g`; whenever the next step will not rebuild (twice the displacement since the
    last rebuild within 0.9 skin), compare its pair signature, walked through the lists, with
    the oracle's brute-force signature of the same state.  Returns the number compared."""
    skin = min(dm / c for dm, c in zip(w.dim, w.cells)) - w.cutoff
    side = np.array(w.dim, np.float64)
    x_in = g.download()["x"].astype(np.float64)
    ref = None
    checked = nb = 0
    for k in range(steps):
        if on_step:
            on_step(k)
        g.step(1)
        nb1 = g.verlet()[0]
        if nb1 > nb:
            ref = x_in            # this step re-binned the positions that entered it
        nb = nb1
        d = g.download()
        x_in = d["x"].astype(np.float64)
        dd = x_in - ref
        dd -= side * np.round(dd / side)
        if 2.0 * np.max(np.linalg.norm(dd, axis=1)) > 0.9 * skin:
            continue              # the next step rebuilds
        gc, gh = g.pair_signature()
        rc, rh = _held_signature(w, d)
        assert np.array_equal(gc, rc), "pair counts differ for %d particles" % int((gc != rc).sum())
        assert np.array_equal(gh, rh)
        checked += 1
    return checked


@pytest.mark.parametrize("name", ["cell_sorting", "bonded"])
def test_pair_list_walk_bitexact(name):
    """Between rebuilds the table variants evaluate the pair lists recorded at the last
    rebuild.  Walked at the current positions while twice the displacement since that
    rebuild is within the skin, the lists give exactly the pairs within the cutoff."""
    w = WORKLOADS[name]()
    assert _walk_and_compare(make_gpu(w), w, 14) >= 3


def test_dense_cells_past_the_list_estimate():
    """A block at twice the mean density overflows the first list size (estimated from the
    mean density): its cells are tested pair by pair, the lists grow at the next call, and
    after the next rebuild they hold those cells too.  Pair sets stay exact throughout."""
    w = configs.verlet(configs.cell_sorting(n=4000, side=20.0, seed=31), skin=0.3)
    rng = np.random.default_rng(5)

    def lattice(lo, hi, a):
        g1 = np.arange(lo, hi, a, dtype=np.float32)
        return np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), axis=-1).reshape(-1, 3)

    block = lattice(2.5, 14.0, 1.0)                     # 12^3 at spacing r0
    sparse = lattice(0.8, 20.0, 20.0 / 12)
    sparse = sparse[np.any((sparse < 1.5) | (sparse > 14.5), axis=1)]
    x = np.concatenate([block, sparse])
    x = x + rng.uniform(-0.05, 0.05, size=x.shape).astype(np.float32)
    n = len(x)
    w = dataclasses.replace(w, x=configs.in_box(x, w.dim[0]), type=w.type[:n], radius=w.radius[:n],
                            imass=w.imass[:n])
    w = dataclasses.replace(_relaxed(w, steps=30), dt=0.0005)   # several steps between rebuilds
    g = make_gpu(w)

    def force_rebuild(k):
        if k == 4:   # re-setting a wall re-lays the arena out: every Verlet simulation rebuilds
            g.set_boundary(0, abi.BOUNDARY_PERIODIC)

    assert _walk_and_compare(g, w, 10, force_rebuild) >= 4


def test_full_size_list_walk_equals_candidate_tests():
    """2.0M-particle LJ fluid in Verlet mode: at every step that does not rebuild, the pair
    set walked through the lists equals the one the candidate tests find (signature of every
    particle), and the engine's trajectory with lists stays with the one without."""
    w = configs.verlet(configs.lj_fluid(n=2_000_000), skin=0.2)
    g = make_gpu(w)
    h = make_gpu(w)
    h.set_pair_lists(False)
    for _ in range(3):
        g.step(4)
        h.step(4)
    rb = g.verlet()[0]
    assert rb == h.verlet()[0]
    gc, gh = g.pair_signature()        # walks the lists (no rebuild is pending: 2 maxdx < skin)
    g.set_pair_lists(False)
    cc, ch = g.pair_signature()        # candidate tests on the same state
    assert np.array_equal(gc, cc) and np.array_equal(gh, ch)
    assert int(gc.sum()) // 2 > 50_000_000
    dev = _dev(g.download()["x"], h.download()["x"], w.dim)
    assert dev.max() < 1e-3


def test_membership_change_forces_a_rebuild():
    """Adding a simulation to a batch re-lays the arena out, which rebuilds every Verlet member
    at the next step (cells, reference positions and pair lists are taken afresh).  The member
    then follows the oracle with a rebuild forced at the same step."""
    w = configs.verlet(configs.cell_sorting(n=2500, side=17.0, seed=41, random_force=(0.0, 2.0, 1)), skin=0.3)
    other = configs.cell_sorting(n=900, side=12.5, seed=42)
    b = Batch(w.max_type, w.nr_species)
    s = b.add_sim(w.desc())
    b._keep.extend(setup_model(s, w))
    o = make_oracle(w)
    b.step(6)
    o.step(6)
    assert s.verlet()[0] == o.verlet()[0]
    s2 = b.add_sim(other.desc())
    b._keep.extend(setup_model(s2, other))
    o.set_boundary(0, abi.BOUNDARY_PERIODIC)     # the oracle's way to force the next step's rebuild
    before = s.verlet()[0]
    b.step(1)
    o.step(1)
    assert s.verlet()[0] == before + 1 == o.verlet()[0]
    b.step(5)
    o.step(5)
    assert s.verlet()[0] == o.verlet()[0]
    a, r = s.download(), o.download()
    assert np.array_equal(a["cell"], r["cell"])
    dev = _dev(a["x"], r["x"], w.dim)
    assert dev.max() < 2e-3 and np.percentile(dev, 99) < 1e-4
