"""Explicit pair lists: the GPU's interacting pairs (tfg_pair_list, recorded by the pair
kernels' own decision) against the pairs the oracle's restatement of runner_dopair /
runner_doself records (tf_runner_dopair.cpp:72-819), as sorted (lower id, higher id) lists.
Every kernel form is covered: the tiled kernel at each work split, the home-outer kernel,
the deterministic stencil kernel, and the overflow pass (crowded cells)."""
import numpy as np
import pytest

from helpers import make_gpu, make_oracle, small_bonded, small_dpd
from tfg import abi, configs

pytestmark = pytest.mark.gpu


def _oracle_pairs(w):
    o = make_oracle(w)
    o.record_pairs(True)
    o.force_only()
    p = np.sort(o.pairs().astype(np.int32), axis=1)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


CASES = {
    "cell_sorting": lambda: configs.cell_sorting(),
    "bonded": lambda: small_bonded(),
    "dpd": lambda: small_dpd(),
    "crowded": lambda: configs.cell_sorting(n=40000, side=20.0, seed=22),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("form", ["split1", "split7", "home", "deterministic"])
def test_pair_list_equals_oracle(name, form):
    w = CASES[name]()
    if name == "crowded" and form == "split7":
        pytest.skip("one work split suffices for the overflow pass")
    g = make_gpu(w)
    if form == "deterministic":
        g.set_deterministic(True)
    else:
        g.set_split({"split1": 1, "split7": 7, "home": abi.PAIR_HOME_OUTER}[form])
    g.force_only()
    gp = g.pair_list()
    op = _oracle_pairs(w)
    assert gp.shape == op.shape, "%s/%s: %d pairs on the GPU, %d in the oracle" % (name, form, len(gp), len(op))
    assert np.array_equal(gp, op), name
