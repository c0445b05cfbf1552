"""Flux kinds and flux substeps on the CUDA path against the oracle: Fick, secrete and
uptake with decay between two particle types, with one species (staged in the tiled pair
pass) and with two or three species (the tiled pass reads them from the particle arrays and
adds their increments there), in the deterministic pass as well, and nr_fluxsteps > 1
(flux-only substep passes)."""
import numpy as np
import pytest

from helpers import FORCE_RTOL, force_error, make_gpu, make_oracle, small_dpd
from tfg import abi, configs

pytestmark = pytest.mark.gpu


def _flux(kind, ta, tb, ia, ib, coef, decay=0.0, target=0.0, cutoff=0.0):
    f = abi.Flux()
    f.kind, f.type_a, f.type_b, f.index_a, f.index_b = kind, ta, tb, ia, ib
    f.coef, f.decay, f.target, f.cutoff = coef, decay, target, cutoff
    return f


def _mixed(nspec, nfs, n=1500, seed=41):
    w = configs.cell_sorting(n=n, side=12.0, seed=seed)
    rng = np.random.default_rng(seed)
    w.nr_species = nspec
    w.species = rng.uniform(0.0, 2.0, size=(n, nspec)).astype(np.float32)
    w.nr_fluxsteps = nfs
    w.fluxes = [(0, 0, _flux(abi.FLUX_FICK, 0, 0, 0, 0, 0.5)),
                (0, 1, _flux(abi.FLUX_SECRETE, 0, 1, 0, nspec - 1, 0.3, decay=0.1, target=0.8, cutoff=2.5)),
                (0, 1, _flux(abi.FLUX_UPTAKE, 0, 1, nspec - 1, 0, 0.4, decay=0.05, target=1.5))]
    return w


def _q_err(a, b):
    scale = np.maximum(np.abs(b), 1e-3 * np.abs(b).max() + 1e-30)
    return float(np.max(np.abs(a - b) / scale))


@pytest.mark.parametrize("nspec,deterministic", [(1, False), (2, False), (2, True)])
def test_flux_kinds_increments_match_oracle(nspec, deterministic):
    w = _mixed(nspec, 1)
    g, o = make_gpu(w), make_oracle(w)
    g.set_deterministic(deterministic)
    g.force_only()
    o.force_only()
    a, b = g.download(), o.download()
    assert force_error(a["f"], b["f"], o.fmag()) < FORCE_RTOL
    assert _q_err(a["q"], b["q"]) < 1e-4


@pytest.mark.parametrize("nspec,nfs", [(1, 2), (2, 3)])
def test_flux_substeps_trajectory_matches_oracle(nspec, nfs):
    w = _mixed(nspec, nfs)
    g, o = make_gpu(w), make_oracle(w)
    g.step(4)
    o.step(4)
    a, b = g.download(), o.download()
    assert np.max(np.abs(a["species"] - b["species"])) < 1e-4
    side = np.array(w.dim, np.float32)
    d = a["x"] - b["x"]
    d -= side * np.round(d / side)
    assert np.max(np.abs(d)) < 1e-3


def test_three_species_droplets_match_oracle():
    """The three-species DPD droplets (Fick on each species, one with decay) at 20,000
    particles: flux increments and forces of one pass, then species after three steps with
    two flux substeps each."""
    w = configs.dpd_droplets_species(n=20_000, side=40.0 * 0.2 ** (1.0 / 3.0), radius=12.0 * 0.2 ** (1.0 / 3.0))
    g, o = make_gpu(w), make_oracle(w)
    g.force_only()
    o.force_only()
    a, b = g.download(), o.download()
    assert _q_err(a["q"], b["q"]) < 1e-4
    assert force_error(a["f"], b["f"], o.fmag()) < FORCE_RTOL
    w.nr_fluxsteps = 2
    g, o = make_gpu(w), make_oracle(w)
    g.step(3)
    o.step(3)
    a, b = g.download(), o.download()
    assert np.max(np.abs(a["species"] - b["species"])) < 1e-4


def test_same_type_secrete_and_uptake_one_pass():
    """Secrete and uptake between two species of particles of one type (20,000 DPD
    droplets): such a flux acts from each pair's first particle to its second, in the
    reference's pair orientation, which within a cell follows the particles' order there.
    Both engines hold the particles of a cell in id order after loading, so one pass must
    agree.  (After particles migrate the reference's cell order is its migration order and
    this engine's is id order again, so trajectories of such fluxes are not compared.)"""
    w = configs.dpd_droplets_species(n=20_000, side=40.0 * 0.2 ** (1.0 / 3.0), radius=12.0 * 0.2 ** (1.0 / 3.0))
    w.fluxes = [w.fluxes[0], (0, 0, _flux(abi.FLUX_SECRETE, 0, 0, 1, 2, 0.3, decay=0.05, target=0.5, cutoff=1.0)),
                (0, 0, _flux(abi.FLUX_UPTAKE, 0, 0, 2, 0, 0.1, target=1.0, cutoff=1.0))]
    g, o = make_gpu(w), make_oracle(w)
    g.force_only()
    o.force_only()
    assert _q_err(g.download()["q"], o.download()["q"]) < 1e-4


def test_dpd_flux_substeps_match_oracle():
    w = small_dpd()
    w.nr_fluxsteps = 4
    g, o = make_gpu(w), make_oracle(w)
    g.step(3)
    o.step(3)
    a, b = g.download(), o.download()
    assert np.max(np.abs(a["species"] - b["species"])) < 1e-4
    assert abs(float(a["species"].sum()) - float(b["species"].sum())) < 1e-3
