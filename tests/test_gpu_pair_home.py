"""The home-particle-outer pair kernel (split TFG_PAIR_HOME_OUTER) against the oracle.

Same bar as the tiled kernel: the interacting-pair set bit-exact (per-particle partner
count and id hash, and explicit pairs for one case), forces and number densities within
FORCE_RTOL normalised, energies within 1e-4.  The cases exercise each path of the kernel:
the self task with one and several 32-particle blocks, neighbourhoods staged in several
chunks, cells too crowded for staging (overflow pass), non-periodic walls with wall
potentials, a batch of uneven simulations, and Verlet mode without pair lists (particles
outside their cells)."""
import numpy as np
import pytest

import oracle as O
from helpers import FORCE_RTOL, force_error, make_gpu, make_oracle, small_bonded, small_cell_sorting
from tfg import abi, configs
from tfg.configs import PotSpec
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu

HOME = abi.PAIR_HOME_OUTER


def _walls():
    w = configs.cell_sorting(n=2500, side=15.0, seed=51)
    w.boundaries = [(0, abi.BOUNDARY_FREESLIP, (0, 0, 0), 1.0, 0.5), (1, abi.BOUNDARY_FREESLIP, (0, 0, 0), 1.0, 0.5)]
    morse = PotSpec("morse", dict(d=1.0, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True))
    w.wall_pots = [(0, 0, morse), (0, 1, morse), (1, 0, morse), (1, 1, morse)]
    return w


CASES = {
    "cell_sorting": lambda: configs.cell_sorting(),                  # 4,000 in 6^3 cells, ~18 per cell
    "cell_sorting_small": lambda: small_cell_sorting(),              # 300 in 3^3 cells
    "bonded": lambda: small_bonded(),                                # 8,000 LJ particles in chains
    # ~60 per cell: several home blocks, neighbourhoods staged in chunks
    "dense": lambda: configs.cell_sorting(n=13000, side=20.0, seed=21),
    # ~185 per cell: every home cell and neighbour together overflow the staging and go to
    # the overflow pass
    "crowded": lambda: configs.cell_sorting(n=40000, side=20.0, seed=22),
    "walls": _walls,
}


@pytest.fixture(params=sorted(CASES))
def case(request):
    return request.param, CASES[request.param]()


def _gpu(w):
    g = make_gpu(w)
    g.set_split(HOME)
    return g


def test_home_pair_set_bitexact(case):
    name, w = case
    g = _gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc), "%s: pair counts differ for %d particles" % (name, int((gc != oc).sum()))
    assert np.array_equal(gh, oh), name


def test_home_forces_density_energy_match_oracle(case):
    name, w = case
    g = _gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    a, b = g.download(), o.download()
    err = force_error(a["f"], b["f"], o.fmag())
    assert err < FORCE_RTOL, "%s: normalised force error %.3g" % (name, err)
    dens_err = np.max(np.abs(a["density"] - b["density"]) / np.abs(b["density"]))
    assert dens_err < FORCE_RTOL, name
    rg, ro = g.reductions(), o.reductions()
    scale = max(abs(ro.epot_nonbond), 1.0)
    assert abs(rg.epot_nonbond - ro.epot_nonbond) / scale < 1e-4, name
    assert abs(rg.virial - ro.virial) / max(abs(ro.virial), 1.0) < 1e-4, name


def test_home_explicit_pairs_match_oracle_record():
    """The pair set against the oracle's explicit pair list (its window walk's recorded
    pairs), not against the oracle's own signature accumulation."""
    w = small_cell_sorting(n=600, side=11.0, seed=9)
    g = _gpu(w)
    o = make_oracle(w)
    o.record_pairs(True)
    g.force_only()
    o.force_only()
    pr = o.pairs().astype(np.int64)
    cnt = np.zeros(w.n, np.int64)
    np.add.at(cnt, pr[:, 0], 1)
    np.add.at(cnt, pr[:, 1], 1)
    gc, gh = g.pair_signature()
    assert np.array_equal(gc, cnt)
    eh = np.zeros(w.n, np.uint64)
    np.add.at(eh, pr[:, 0], O.sig_mix(pr[:, 1]))
    np.add.at(eh, pr[:, 1], O.sig_mix(pr[:, 0]))
    assert np.array_equal(gh, (eh & 0xFFFFFFFF).astype(np.uint32))


def test_home_batch_members_match_alone():
    ws = [configs.cell_sorting(n=300, side=10.0, seed=11),
          configs.cell_sorting(n=2500, side=17.0, depth_ab=0.4, seed=12, random_force=(0.0, 0.1, 1)),
          configs.cell_sorting(n=900, side=12.5, depth_ab=1.7, seed=13),
          configs.cell_sorting(n=6000, side=22.9, seed=14)]
    b = Batch(ws[0].max_type, ws[0].nr_species)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.set_split(HOME)
    b.force_only()
    for s, w in zip(sims, ws):
        o = make_oracle(w)
        o.force_only()
        err = force_error(s.download()["f"], o.download()["f"], o.fmag())
        assert err < FORCE_RTOL, "%s: %.3g" % (w.name, err)


def test_home_trajectory_matches_tiled_kernel():
    """Ten steps with the home kernel stay within the trajectory bar of the tiled kernel."""
    w = configs.cell_sorting(n=3000, side=18.0, seed=31, random_force=(0.0, 0.1, 1))
    g1 = _gpu(w)
    g2 = make_gpu(w)
    g2.set_split(1)
    g1.step(10)
    g2.step(10)
    a, b = g1.download(), g2.download()
    side = np.array(w.dim, np.float32)
    d = a["x"] - b["x"]
    d -= side * np.round(d / side)
    assert np.max(np.abs(d)) < 1e-3
    assert np.mean(a["cell"] != b["cell"]) < 1e-3


def test_home_verlet_without_lists():
    """Verlet mode with the pair lists off: between rebuilds particles sit outside their
    cells, and the home kernel must still find exactly the oracle's pairs."""
    w = configs.verlet(configs.lj_fluid(n=4000, density=0.8), skin=0.3)
    g = make_gpu(w)
    g.set_pair_lists(False)
    g.set_split(HOME)
    o = make_oracle(w)
    for _ in range(3):
        g.step(1)
        o.step(1)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
    assert force_error(g.download()["f"], o.download()["f"], o.fmag()) < FORCE_RTOL
