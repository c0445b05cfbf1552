"""Known-answer tests of the oracle's flux path beyond Fick diffusion: the secrete and
uptake kinds and decay (flux_eval_ex, tf_flux_eval.h:32-103), and flux substeps
(nr_fluxsteps > 1: flux-only passes plus Fluxes_integrate before the step's force pass,
tf_engine_advance.cpp:314-323; dt_flux = dt / nr_fluxsteps, tfSimulator.cpp:653)."""
import numpy as np

import oracle as O
from tfg import abi


def _flux(kind, ta, tb, coef, decay=0.0, target=0.0, cutoff=1.0):
    f = abi.Flux()
    f.kind, f.type_a, f.type_b, f.index_a, f.index_b = kind, ta, tb, 0, 0
    f.coef, f.decay, f.target, f.cutoff = coef, decay, target, cutoff
    return f


def _pair(species, types, flux, ti, tj, nfs=1, dt=0.005):
    d = abi.engine_desc((0, 0, 0), (20.0,) * 3, (20,) * 3, 1.0, dt, max_type=2, nr_species=1,
                        nr_fluxsteps=nfs)
    e = O.OracleEngine(d, O.MODE_NO_DENSITY)
    for t in range(2):
        e.set_type(t, abi.NEWTONIAN)
    e.add_flux(ti, tj, flux)
    e.load(np.array([[5.0, 5.0, 5.0], [5.5, 5.0, 5.0]], np.float32), type=np.array(types, np.int32),
           species=np.array(species, np.float32).reshape(2, 1))
    return e


TERM = (1 - 0.5 / 1.0) ** 2   # (1 - r/cutoff)^2 at r = 0.5


def test_fick_substeps_closed_form_and_conservation():
    dt, nfs = 0.005, 3
    e = _pair([1.0, 0.0], [0, 0], _flux(abi.FLUX_FICK, 0, 0, 0.5), 0, 0, nfs=nfs, dt=dt)
    e.step(1)
    s = e.download()["species"][:, 0]
    dtf = np.float32(dt) / np.float32(nfs)
    a, b = np.float32(1.0), np.float32(0.0)
    for _ in range(nfs):
        q = np.float32(TERM * 0.5) * (a - b)
        a, b = a - dtf * q, b + dtf * q
    assert abs(s[0] - a) < 1e-6 and abs(s[1] - b) < 1e-6
    assert abs(s.sum() - 1.0) < 1e-6


def test_secrete_moves_excess_above_target():
    k, target, dt = 0.5, 0.5, 0.005
    e = _pair([2.0, 0.0], [0, 1], _flux(abi.FLUX_SECRETE, 0, 1, k, target=target), 0, 1, dt=dt)
    e.step(1)
    s = e.download()["species"][:, 0]
    q = TERM * max(0.0, k * (2.0 - target))
    assert abs(s[0] - (2.0 - dt * q)) < 1e-6
    assert abs(s[1] - dt * q) < 1e-6
    # below the target nothing moves
    e = _pair([0.4, 0.0], [0, 1], _flux(abi.FLUX_SECRETE, 0, 1, k, target=target), 0, 1, dt=dt)
    e.step(1)
    assert np.allclose(e.download()["species"][:, 0], [0.4, 0.0], atol=1e-7)


def test_uptake_and_decay():
    k, target, decay, dt = 0.5, 1.0, 0.2, 0.005
    e = _pair([1.0, 0.2], [0, 1], _flux(abi.FLUX_UPTAKE, 0, 1, k, decay=decay, target=target), 0, 1, dt=dt)
    e.force_only()
    q_inc = e.download()["q"][:, 0]
    q = TERM * max(0.0, k * (target - 0.2) * 1.0)
    assert abs(q_inc[0] - (-q - decay / 2 * 1.0)) < 1e-6
    assert abs(q_inc[1] - (q - decay / 2 * 0.2)) < 1e-6
