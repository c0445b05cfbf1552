"""Force error of the FP32 GPU pass against an FP64 evaluation, stated per configuration.

The oracle's FP64 mode evaluates the same tables and the same pair set in double precision
(potential_eval_ex, dpd_eval, W and the bonded terms with FP64 arithmetic, FP32 tables as
the reference stores them), so the difference isolates the GPU's FP32 evaluation and
summation order.  For every configuration the maximum and the 99th percentile of the
per-particle normalised error |f_gpu - f_fp64| / sum_j |f_ij| are printed (run pytest with
-s to see them) and the maximum must stay below FORCE_RTOL = 1e-5:
- cell sorting, 4,000 particles (the full configuration);
- DPD droplets with Fickian flux, 100,000 particles (full), noise on;
- bonded fluid, 2,000,000 particles in chains with bonds and angles (full);
- the batched ensemble: every 16th of its 256 simulations, in one batch.
"""
import os

import numpy as np
import pytest

import oracle as O
from helpers import FORCE_RTOL, make_gpu, make_oracle
from tfg import abi, configs
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def _errors(f_gpu, f64, fmag):
    d = np.linalg.norm(np.asarray(f_gpu, np.float64) - f64[:, :3], axis=1)
    e = d / np.maximum(fmag, 1e-30)
    return float(e.max()), float(np.percentile(e, 99))


def _single(w):
    g = make_gpu(w)
    o32 = make_oracle(w, threads=THREADS)
    o64 = make_oracle(w, O.MODE_FP64, threads=THREADS)
    g.force_only()
    o32.force_only()
    o64.force_only()
    return _errors(g.download()["f"], o64.forces_f64(), o32.fmag())


CONFIGS = {
    "cell_sorting_4000": lambda: configs.cell_sorting(),
    "dpd_droplets_100k": lambda: configs.dpd_droplets(),
    "bonded_fluid_2M": lambda: configs.bonded_fluid(),
}


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_fp64_error_per_configuration(name):
    mx, p99 = _single(CONFIGS[name]())
    print("FP64 force error %s: max %.3g, p99 %.3g" % (name, mx, p99))
    assert mx < FORCE_RTOL


@pytest.mark.parametrize("split", [1, abi.PAIR_HOME_OUTER])
def test_fp64_error_ensemble_sample(split):
    ws = configs.ensemble()[::16]
    b = Batch(ws[0].max_type, ws[0].nr_species)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.set_split(split)
    b.force_only()
    worst, p99s = 0.0, []
    for s, w in zip(sims, ws):
        o32 = make_oracle(w, threads=THREADS)
        o64 = make_oracle(w, O.MODE_FP64, threads=THREADS)
        o32.force_only()
        o64.force_only()
        mx, p99 = _errors(s.download()["f"], o64.forces_f64(), o32.fmag())
        worst = max(worst, mx)
        p99s.append(p99)
    print("FP64 force error ensemble (16 of 256, split %d): max %.3g, p99 %.3g" % (split, worst, max(p99s)))
    assert worst < FORCE_RTOL
