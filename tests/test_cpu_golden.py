"""The oracle reproduces the committed golden fixtures (tests/golden/*.npz, written by
tests/golden/make_golden.py from the oracle itself): cells, cell-relative positions and
pair signatures exactly; forces, densities, flux increments and short trajectories to
within a few FP32 ulps (the tables come from libm, which may differ between hosts)."""
import os

import numpy as np
import pytest

from golden.make_golden import cases, oracle_engine

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def _close(a, b, rtol=2e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b), 1e-3 * (np.abs(b).max() + 1e-30))
    return float(np.max(np.abs(a - b) / scale)) if a.size else 0.0


@pytest.mark.parametrize("name", sorted(cases()))
def test_oracle_matches_golden(name):
    make, steps = cases()[name]
    w = make()
    g = _load(name)
    assert np.array_equal(w.x, g["x_in"]) and np.array_equal(w.type, g["type_in"])
    e = oracle_engine(w)
    d = e.download()
    assert np.array_equal(d["cell"], g["load_cell"])
    assert np.array_equal(d["xrel"].view(np.uint32), g["load_xrel"].view(np.uint32))
    e.force_only()
    cnt, hsh = e.signature()
    assert np.array_equal(cnt, g["sig_count"]) and np.array_equal(hsh, g["sig_hash"])
    d = e.download()
    assert _close(d["f"], g["force"]) < 1e-5
    assert _close(d["density"], g["density"]) < 1e-6
    if "q" in g:
        assert _close(d["q"], g["q"]) < 1e-5
    e2 = oracle_engine(w)
    e2.step(int(g["steps"]))
    d = e2.download()
    assert np.max(np.abs(d["x"] - g["traj_x"])) < 1e-4
    assert np.mean(d["cell"] != g["traj_cell"]) < 1e-2
