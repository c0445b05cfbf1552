"""The CUDA path at the configurations' full sizes.

The 100,000-particle DPD droplets and the 2,000,000-particle bonded fluid are compared
with the threaded oracle on one force pass (pair sets bit-exact, forces within FORCE_RTOL).
Size-independent properties are checked over several steps, alone or on the 256-simulation
ensemble:
- Newton's third law leaves no net force;
- binning keeps every cell-relative position inside its cell and the particles sorted by cell;
- Fickian flux conserves the species total;
- a sample of the batched ensemble equals the same simulations run alone."""
import os

import numpy as np
import pytest

from helpers import FORCE_RTOL, force_error, make_gpu, make_oracle
from tfg import configs
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.mark.parametrize("name", ["dpd_droplets", "bonded_fluid"])
def test_full_size_force_pass_matches_oracle(name):
    w = configs.dpd_droplets() if name == "dpd_droplets" else configs.bonded_fluid()
    g, o = make_gpu(w), make_oracle(w, threads=THREADS)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
    a, b = g.download(), o.download()
    assert force_error(a["f"], b["f"], o.fmag()) < FORCE_RTOL
    if w.nr_species:
        scale = np.maximum(np.abs(b["q"]), 1e-3 * np.abs(b["q"]).max() + 1e-30)
        assert np.max(np.abs(a["q"] - b["q"]) / scale) < 1e-4


def test_full_size_newton_third_law():
    w = configs.bonded_fluid()
    g = make_gpu(w)
    g.force_only()
    f = g.download()["f"].astype(np.float64)
    total = f.sum(axis=0)
    scale = np.abs(f).sum(axis=0)
    assert np.all(np.abs(total) <= 1e-5 * scale)


def test_full_size_binning_invariants_and_conservation():
    w = configs.dpd_droplets()
    g = make_gpu(w)
    s0 = g.download()["species"].astype(np.float64).sum()
    g.step(20)
    d = g.download()
    h = np.array(w.dim, np.float32) / np.array(w.cells, np.float32)
    assert np.all(d["xrel"] >= 0) and np.all(d["xrel"] < h)
    c = np.array(w.cells)
    loc = np.stack([d["cell"] // (c[1] * c[2]), (d["cell"] // c[2]) % c[1], d["cell"] % c[2]], axis=1)
    orig = loc * h
    assert np.allclose(orig + d["xrel"], d["x"], atol=1e-4)
    s1 = d["species"].astype(np.float64).sum()
    assert abs(s1 - s0) <= 1e-5 * max(1.0, abs(s0))
    r = g.reductions()
    assert r.steps == 20 and abs(r.species_total[0] - s1) <= 1e-4 * max(1.0, abs(s1))


def test_full_ensemble_sample_equals_alone():
    ws = configs.ensemble()
    b = Batch(2, 0)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.step(5)
    for k in (0, 97, 255):
        g = make_gpu(ws[k])
        g.step(5)
        a, r = sims[k].download(), g.download()
        assert np.array_equal(a["cell"], r["cell"]) or np.mean(a["cell"] != r["cell"]) < 1e-3
        side = np.array(ws[k].dim, np.float32)
        dx = a["x"] - r["x"]
        dx -= side * np.round(dx / side)
        assert np.max(np.abs(dx)) < 1e-3
