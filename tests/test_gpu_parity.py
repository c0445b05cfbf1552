"""Parity of the CUDA path (called through the C ABI) with the CPU oracle.

Bar: cell membership, cell-relative positions and interacting-pair sets bit-exact;
per-particle forces, number densities and flux increments within FORCE_RTOL (1e-5)
normalised by the sum of contribution magnitudes; trajectories within the stated
tolerance."""
import numpy as np
import pytest

import oracle as O
from helpers import FORCE_RTOL, force_error, make_gpu, make_oracle, small_bonded, small_cell_sorting, small_dpd
from tfg import abi, configs
from tfg.engine import Batch, Engine, TfgError, setup_model

pytestmark = pytest.mark.gpu

WORKLOADS = {
    "cell_sorting": lambda: configs.cell_sorting(),            # 4,000 particles, 6^3 cells
    "cell_sorting_small": lambda: small_cell_sorting(),        # 300 particles, 3^3 cells
    "dpd": lambda: small_dpd(),                                # 4,000 DPD particles with flux
    "bonded": lambda: small_bonded(),                          # 8,000 LJ particles in chains
}


@pytest.fixture(params=sorted(WORKLOADS))
def wl(request):
    return request.param, WORKLOADS[request.param]()


def test_load_binning_bitexact(wl):
    name, w = wl
    g = make_gpu(w)
    o = make_oracle(w)
    a, b = g.download(), o.download()
    assert np.array_equal(a["cell"], b["cell"])
    assert np.array_equal(a["xrel"].view(np.uint32), b["xrel"].view(np.uint32))


def test_pair_set_bitexact(wl):
    name, w = wl
    g = make_gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc), "pair counts differ for %d particles" % int((gc != oc).sum())
    assert np.array_equal(gh, oh)


def test_forces_density_flux_match_oracle(wl):
    name, w = wl
    g = make_gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    a, b = g.download(), o.download()
    err = force_error(a["f"], b["f"], o.fmag())
    assert err < FORCE_RTOL, "normalised force error %.3g" % err
    dens_err = np.max(np.abs(a["density"] - b["density"]) / np.abs(b["density"]))
    assert dens_err < FORCE_RTOL
    if w.nr_species:
        q_scale = np.maximum(np.abs(b["q"]), 1e-3 * np.abs(b["q"]).max() + 1e-30)
        assert np.max(np.abs(a["q"] - b["q"]) / q_scale) < 1e-4


@pytest.mark.parametrize("split", [1, 2, 7, 14])
def test_every_work_split_matches(split):
    """Each work split of the tiled pass (warps per home cell) gives the same pair set and
    forces within tolerance."""
    w = configs.cell_sorting()
    g = make_gpu(w)
    g.set_split(split)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
    assert force_error(g.download()["f"], o.download()["f"], o.fmag()) < FORCE_RTOL


@pytest.mark.parametrize("tuple_", [(1, 4, 1), (2, 8, 2), (7, 4, 4), (14, 8, 4), (1, 4, 8)])
def test_every_tuning_tuple_matches(tuple_):
    """Warps per CTA (8, or 4 for tabulated potentials) and work items per grab change only
    the launch shape: the pair set stays bit-exact and the forces within tolerance."""
    w = configs.cell_sorting()
    g = make_gpu(w)
    g.set_tuning(*tuple_)
    assert g.tuning() == tuple_
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
    assert force_error(g.download()["f"], o.download()["f"], o.fmag()) < FORCE_RTOL


def test_autotune_picks_a_valid_tuple():
    w = configs.cell_sorting()
    g = make_gpu(w)
    split = g.autotune()
    t = g.tuning()
    assert t[0] == split and split in (1, 2, 7, 14, abi.PAIR_HOME_OUTER)
    assert t[1] in (4, 8) and t[2] in (1, 2, 4)


def test_autotune_leaves_state_unchanged():
    w = small_dpd()
    g = make_gpu(w)
    before = g.download()
    split = g.autotune()
    assert split in (1, 2, 7, 14)
    after = g.download()
    for k in ("x", "v", "species", "q", "cell"):
        assert np.array_equal(before[k], after[k]), k


def test_forces_vs_fp64_oracle(wl):
    """The FP32 GPU forces against the FP64 evaluation of the same tables and pair set."""
    name, w = wl
    g = make_gpu(w)
    o32 = make_oracle(w)
    o64 = make_oracle(w, O.MODE_FP64)
    g.force_only()
    o32.force_only()
    o64.force_only()
    err = force_error(g.download()["f"], o64.forces_f64()[:, :3], o32.fmag())
    assert err < FORCE_RTOL, "normalised force error vs FP64 %.3g" % err


def test_integrator_and_migration_bitexact_under_external_forces():
    """With no pair interactions the force is exactly force_i, so positions, velocities
    and cell membership must stay bit-identical to the oracle over many steps, including
    clamped displacements and cell migrations (tf_engine_advance.cpp:140-247)."""
    rng = np.random.default_rng(11)
    n = 5000
    for dyn in (abi.OVERDAMPED, abi.NEWTONIAN):
        w = configs.cell_sorting(n=n, seed=21)
        w.pots = {}
        w.dynamics = [dyn, dyn]
        fi = rng.normal(0, 300.0, size=(n, 3)).astype(np.float32)
        fi[::7] *= 1e4   # clamped
        w.v = rng.normal(0, 5.0, size=(n, 3)).astype(np.float32)
        g = Engine(w.desc())
        o = O.OracleEngine(w.desc(), O.MODE_NO_DENSITY)
        for e in (g, o):
            for t in range(2):
                e.set_type(t, dyn, 1.0)
            e.load(w.x, v=w.v, type=w.type, force_i=fi)
        g.step(40)
        o.step(40)
        a, b = g.download(), o.download()
        assert np.array_equal(a["cell"], b["cell"])
        assert np.array_equal(a["xrel"].view(np.uint32), b["xrel"].view(np.uint32))
        assert np.array_equal(a["v"].view(np.uint32), b["v"].view(np.uint32))
        assert g.reductions().migrations == o.reductions().migrations


def test_trajectory_10_steps(wl):
    name, w = wl
    g = make_gpu(w)
    o = make_oracle(w)
    g.step(10)
    o.step(10)
    a, b = g.download(), o.download()
    side = np.array(w.dim, np.float32)
    d = a["x"] - b["x"]
    d -= side * np.round(d / side)
    # The GPU sums forces in another (and run-to-run varying) order than the oracle; close
    # contacts amplify the FP32 rounding differences over the steps.  Bar: every particle
    # within 2e-3, 99% of them within 1e-4.
    dev = np.abs(d).max(axis=1)
    assert dev.max() < 2e-3, "max position deviation %.3g" % dev.max()
    assert np.percentile(dev, 99) < 1e-4, "99th percentile deviation %.3g" % np.percentile(dev, 99)
    assert np.mean(a["cell"] != b["cell"]) < 1e-3
    if w.nr_species:
        assert np.max(np.abs(a["species"] - b["species"])) < 1e-4


def test_reductions_match(wl):
    name, w = wl
    g = make_gpu(w)
    o = make_oracle(w)
    g.step(1)
    o.step(1)
    rg, ro = g.reductions(), o.reductions()
    assert abs(rg.kinetic - ro.kinetic) <= 1e-6 * max(1.0, abs(ro.kinetic))
    assert abs(rg.epot_nonbond - ro.epot_nonbond) <= 1e-4 * max(1.0, abs(ro.epot_nonbond))
    assert abs(rg.epot_bond - ro.epot_bond) <= 1e-4 * max(1.0, abs(ro.epot_bond))
    assert abs(rg.epot_angle - ro.epot_angle) <= 1e-4 * max(1.0, abs(ro.epot_angle))
    for s in range(w.nr_species):
        assert abs(rg.species_total[s] - ro.species_total[s]) <= 1e-5 * max(1.0, abs(ro.species_total[s]))
    assert rg.migrations == ro.migrations or abs(rg.migrations - ro.migrations) <= 2


def test_dpd_reference_random_mode_matches():
    w = small_dpd()
    w.flags = abi.ENGINE_DPD_REFERENCE_RANDOM
    g = make_gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    assert force_error(g.download()["f"], o.download()["f"], o.fmag()) < FORCE_RTOL


def test_random_force_matches_oracle():
    w = configs.cell_sorting(n=2000, random_force=(0.0, 0.1, 1))
    g = make_gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    assert force_error(g.download()["f"], o.download()["f"], o.fmag()) < FORCE_RTOL


def test_invalid_configuration_rejected():
    bad = abi.engine_desc((0, 0, 0), (10, 10, 10), (2, 2, 2), 1.0, 0.01)
    with pytest.raises(TfgError) as ei:
        Engine(bad)
    assert ei.value.code == abi.TFG_E_INVAL
    # cell edge below the cutoff (span 2) is not supported
    with pytest.raises(TfgError):
        Engine(abi.engine_desc((0, 0, 0), (10, 10, 10), (8, 8, 8), 2.0, 0.01))
    g = Engine(abi.engine_desc((0, 0, 0), (10, 10, 10), (3, 3, 3), 3.0, 0.01, max_type=1))
    with pytest.raises(TfgError) as ei:
        g.load(np.zeros((4, 3), np.float32), type=np.array([0, 1, 0, 0], np.int32))
    assert ei.value.code == abi.TFG_E_INVAL
    with pytest.raises(TfgError) as ei:
        g.step(1)
    assert ei.value.code == abi.TFG_E_STATE


def test_empty_and_ragged_cells():
    """Few particles in many cells (most cells empty) and all particles in one cell."""
    d = abi.engine_desc((0, 0, 0), (30, 30, 30), (10, 10, 10), 3.0, 0.005, max_type=1)
    from tfg import Potential
    p = Potential.morse(d=1.0, a=5.0, r0=1.0, min=0.01, max=3.0)
    rng = np.random.default_rng(3)
    for x in (rng.uniform(0, 30, size=(7, 3)), rng.uniform(10.0, 12.9, size=(300, 3))):
        x = x.astype(np.float32)
        g = Engine(d)
        o = O.OracleEngine(d)
        for e in (g, o):
            e.set_type(0, abi.OVERDAMPED)
            e.set_potential(0, 0, p.ptr)
            e.load(x)
        g.force_only()
        o.force_only()
        gc, gh = g.pair_signature()
        oc, oh = o.signature()
        assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
        assert force_error(g.download()["f"], o.download()["f"], o.fmag()) < FORCE_RTOL


def test_retune_after_growth_keeps_results():
    """A batch tuned on one small member and then grown more than 4x re-times its work
    split at the next step; the members still equal their alone runs."""
    ws = [configs.cell_sorting(n=600, side=11.0, seed=71)] + \
         [configs.cell_sorting(n=3000, side=18.0, seed=72 + k) for k in range(4)]
    b = Batch(ws[0].max_type, ws[0].nr_species)
    first = b.add_sim(ws[0].desc())
    b._keep.extend(setup_model(first, ws[0]))
    b.step(2)
    t_small = b.tuning()
    sims = [first]
    for w in ws[1:]:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.step(3)
    t_big = b.tuning()
    assert t_big[0] in (1, 2, 7, 14, abi.PAIR_HOME_OUTER) and t_small[0] in (1, 2, 7, 14, abi.PAIR_HOME_OUTER)
    for s, w, steps in zip(sims, ws, [5, 3, 3, 3, 3]):
        g = make_gpu(w)
        g.step(steps)
        side = np.array(w.dim, np.float32)
        d = s.download()["x"] - g.download()["x"]
        d -= side * np.round(d / side)
        assert np.max(np.abs(d)) < 1e-3
