"""A model imported from a FIO file (tfg.fio) runs on the GPU as the oracle runs it: pair set
bit-exact, trajectory at the parity bar, alone and as a member of a batch."""
import os

import numpy as np
import pytest

from helpers import make_gpu, make_oracle
from tfg import fio
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _dev(a, b, dim):
    side = np.array(dim, np.float32)
    d = a - b
    d -= side * np.round(d / side)
    return np.abs(d).max(axis=1)


def test_imported_model_matches_oracle_alone_and_in_a_batch():
    w = fio.load(os.path.join(GOLDEN, "fio_reference_style.json"))
    g = make_gpu(w)
    o = make_oracle(w)
    g.force_only()
    o.force_only()
    gc, gh = g.pair_signature()
    oc, oh = o.signature()
    assert np.array_equal(gc, oc) and np.array_equal(gh, oh)
    g.step(10)
    o.step(10)
    a, b = g.download(), o.download()
    dev = _dev(a["x"], b["x"], w.dim)
    assert dev.max() < 2e-3 and np.percentile(dev, 99) < 1e-4
    bt = Batch(w.max_type, w.nr_species)
    s = bt.add_sim(w.desc())
    bt._keep.extend(setup_model(s, w))
    other = fio.load(os.path.join(GOLDEN, "fio_reference_style.json"))
    other.x = other.x[::-1].copy()
    s2 = bt.add_sim(other.desc())
    bt._keep.extend(setup_model(s2, other))
    bt.step(11)
    alone = make_gpu(w)
    alone.step(11)
    assert _dev(s.download()["x"], alone.download()["x"], w.dim).max() < 1e-3
