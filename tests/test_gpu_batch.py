"""Batches: several independent simulations in one device arena.

Each simulation of a batch must give what it gives alone: the same pair set (bit-exact,
checked against the oracle's recorded pairs), forces within FORCE_RTOL of the oracle, and
trajectories that match running it alone, also after other simulations are added to or
removed from the arena between steps."""
import numpy as np
import pytest

import oracle as O
from helpers import FORCE_RTOL, force_error, make_gpu, make_oracle
from tfg import configs
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu


def _members():
    """Uneven sizes and boxes, distinct seeds and AB depths, random force on some."""
    return [configs.cell_sorting(n=300, side=10.0, seed=11),
            configs.cell_sorting(n=2500, side=17.0, depth_ab=0.4, seed=12, random_force=(0.0, 0.1, 1)),
            configs.cell_sorting(n=900, side=12.5, depth_ab=1.7, seed=13),
            configs.cell_sorting(n=6000, side=22.9, seed=14, random_force=(0.0, 0.1, 1))]


def _batch(ws):
    b = Batch(ws[0].max_type, ws[0].nr_species)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    return b, sims


def _wrap_dev(a, b, dim):
    side = np.array(dim, np.float32)
    d = a - b
    d -= side * np.round(d / side)
    return float(np.max(np.abs(d))) if len(d) else 0.0


def test_batch_pair_sets_bitexact():
    ws = _members()
    b, sims = _batch(ws)
    b.force_only()
    cnt, hsh = b.pair_signature()
    off = 0
    for w in ws:
        o = make_oracle(w)
        o.record_pairs(True)
        o.force_only()
        pr = o.pairs().astype(np.int64) + off
        ec = np.zeros(w.n, np.int64)
        eh = np.zeros(w.n, np.uint64)
        np.add.at(ec, pr[:, 0] - off, 1)
        np.add.at(ec, pr[:, 1] - off, 1)
        np.add.at(eh, pr[:, 0] - off, O.sig_mix(pr[:, 1]))
        np.add.at(eh, pr[:, 1] - off, O.sig_mix(pr[:, 0]))
        assert np.array_equal(cnt[off:off + w.n], ec.astype(np.int32)), w.name
        assert np.array_equal(hsh[off:off + w.n], (eh & 0xFFFFFFFF).astype(np.uint32)), w.name
        off += w.n


def test_batch_forces_match_oracle():
    ws = _members()
    b, sims = _batch(ws)
    b.force_only()
    for w, s in zip(ws, sims):
        o = make_oracle(w)
        o.force_only()
        a, r = s.download(), o.download()
        err = force_error(a["f"], r["f"], o.fmag())
        assert err < FORCE_RTOL, "%s: normalised force error %.3g" % (w.name, err)
        assert np.max(np.abs(a["density"] - r["density"]) / np.abs(r["density"])) < FORCE_RTOL


def test_batch_binning_and_reductions_match_alone():
    ws = _members()
    b, sims = _batch(ws)
    b.step(1)
    for w, s in zip(ws, sims):
        g = make_gpu(w)
        g.step(1)
        a, r = s.download(), g.download()
        assert np.array_equal(a["cell"], r["cell"]), w.name
        ra, rr = s.reductions(), g.reductions()
        assert ra.steps == rr.steps == 1
        assert abs(ra.kinetic - rr.kinetic) <= 1e-6 * max(1.0, abs(rr.kinetic))
        assert abs(ra.epot - rr.epot) <= 1e-5 * max(1.0, abs(rr.epot))
        assert ra.migrations == rr.migrations or abs(ra.migrations - rr.migrations) <= 2


def test_batch_trajectory_matches_alone_and_oracle():
    ws = _members()
    b, sims = _batch(ws)
    b.step(10)
    for w, s in zip(ws, sims):
        o = make_oracle(w)
        o.step(10)
        a, r = s.download(), o.download()
        dev = _wrap_dev(a["x"], r["x"], w.dim)
        assert dev < 1e-3, "%s: max position deviation %.3g" % (w.name, dev)


def test_batch_add_remove_between_steps():
    """Removing and adding simulations re-lays the arena out; the survivors carry on as if alone."""
    ws = _members()
    b, sims = _batch(ws[:3])
    b.step(4)
    b.remove_sim(sims[1])
    late = b.add_sim(ws[3].desc())
    b._keep.extend(setup_model(late, ws[3]))
    assert b.live_count() == 3
    b.step(6)
    for w, s, steps in ((ws[0], sims[0], 10), (ws[2], sims[2], 10), (ws[3], late, 6)):
        o = make_oracle(w)
        o.step(steps)
        a, r = s.download(), o.download()
        assert s.reductions().steps == steps
        dev = _wrap_dev(a["x"], r["x"], w.dim)
        assert dev < 1e-3, "%s: max position deviation %.3g" % (w.name, dev)
    with pytest.raises(Exception):
        sims[1].download()


def test_batch_mixed_dpd_flux_members():
    """Members with DPD, flux and species next to each other (one species, two types)."""
    ws = [configs.dpd_droplets(n=3000, side=12.0, radius=3.5, seed=21),
          configs.dpd_droplets(n=1500, side=10.0, radius=3.0, seed=22)]
    b, sims = _batch(ws)
    b.force_only()
    for w, s in zip(ws, sims):
        o = make_oracle(w)
        o.force_only()
        a, r = s.download(), o.download()
        assert force_error(a["f"], r["f"], o.fmag()) < FORCE_RTOL, w.name
        q_scale = np.maximum(np.abs(r["q"]), 1e-3 * np.abs(r["q"]).max() + 1e-30)
        assert np.max(np.abs(a["q"] - r["q"]) / q_scale) < 1e-4, w.name
