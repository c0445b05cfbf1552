"""Shared test helpers: build the same model into the GPU engine and the CPU oracle,
and compare their outputs with the metrics the parity bar is stated in."""
import numpy as np

import oracle as O
from tfg import configs
from tfg.engine import Engine, setup_model

# Per-particle force tolerance (FP32 vs FP32 oracle), normalised by the sum of the
# magnitudes of the contributions to that particle: |f_gpu - f_ref| / S_i.
FORCE_RTOL = 1e-5


def make_oracle(w, mode=0, threads=1):
    e = O.OracleEngine(w.desc(), mode, threads)
    keep = setup_model(e, w)
    e._keep = keep
    return e


def make_gpu(w):
    e = Engine(w.desc())
    keep = setup_model(e, w)
    e._keep = keep
    return e


def force_error(f_test, f_ref, fmag):
    """max_i |f_test - f_ref| / max(S_i, tiny)."""
    d = np.linalg.norm(np.asarray(f_test, np.float64) - np.asarray(f_ref, np.float64), axis=1)
    s = np.maximum(np.asarray(fmag, np.float64), 1e-30)
    return float(np.max(d / s)) if len(d) else 0.0


def small_cell_sorting(n=300, side=10.0, seed=5):
    return configs.cell_sorting(n=n, side=side, seed=seed)


def small_dpd(n=4000, side=12.0, seed=7):
    return configs.dpd_droplets(n=n, side=side, radius=3.5, seed=seed)


def small_bonded(n=16 * 500, seed=9):
    return configs.bonded_fluid(n=n, seed=seed)
