"""The CUDA path against the committed golden fixtures (tests/golden/*.npz): binning and
pair sets bit-exact, forces within FORCE_RTOL normalised by the per-particle sum of
contribution magnitudes, short trajectories within 1e-3."""
import os

import numpy as np
import pytest

from golden.make_golden import cases
from helpers import FORCE_RTOL, force_error, make_gpu

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(cases()))
def test_gpu_matches_golden(name):
    make, steps = cases()[name]
    w = make()
    g = dict(np.load(os.path.join(HERE, name + ".npz")))
    w.x = g["x_in"]
    w.type = g["type_in"]
    e = make_gpu(w)
    d = e.download()
    assert np.array_equal(d["cell"], g["load_cell"])
    assert np.array_equal(d["xrel"].view(np.uint32), g["load_xrel"].view(np.uint32))
    e.force_only()
    cnt, hsh = e.pair_signature()
    assert np.array_equal(cnt, g["sig_count"]) and np.array_equal(hsh, g["sig_hash"])
    d = e.download()
    assert force_error(d["f"], g["force"], g["fmag"]) < FORCE_RTOL
    e2 = make_gpu(w)
    e2.step(int(g["steps"]))
    d = e2.download()
    side = np.array(w.dim, np.float32)
    dx = d["x"] - g["traj_x"]
    dx -= side * np.round(dx / side)
    assert np.max(np.abs(dx)) < 1e-3
