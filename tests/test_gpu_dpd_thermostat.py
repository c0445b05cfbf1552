"""DPD with the noise on: the fluctuation-dissipation balance on the GPU.

The dissipative and random DPD terms (tf_dpd_eval.h:32-76) form a thermostat only when the
random term is sigma * omega * xi / sqrt(dt) with xi ~ N(0,1) independent per pair and step
and sigma^2 = 2 gamma kT (Espanol & Warren, Europhys. Lett. 30 (1995) 191).  The reference
writes the constant sigma * omega / sqrt(dt) instead (its Gaussian is never used,
tf_dpd_eval.h:64); here xi comes from Philox4x32-10 keyed on (seed, step, pair ids).  With
the droplet workload's physics (alpha 10, gamma 4.5, sigma 3, so kT = sigma^2 / (2 gamma) = 1,
cutoff 1, dt 0.01, mass 1) a homogeneous periodic box must equilibrate at kT = 1:

- Statistical bar: the kinetic temperature averaged over the last half of 600 steps, each
  velocity component's variance, within 0.04 of 1.  The forward-Euler integrator of the
  reference (tf_engine_advance.cpp:170-177) biases the temperature upwards by about
  gamma_eff dt / 2 (a few 1e-3 to 2e-2 at these densities; the oracle gives 1.0085 at
  density 3 and 1.023 at density 6.9); the average over ~30 correlation times of N = 20,000
  particles has a statistical error near 1e-3.
- Momentum: the pair forces are antisymmetric, so the mean velocity stays at its initial
  zero within rounding (|mean| < 5e-3).
- Shape: the velocity components are Gaussian (kurtosis within 0.1 of 3).
- Control: with the reference's constant random term (TFG_ENGINE_DPD_REFERENCE_RANDOM) the
  same box cools far below kT = 1 (to about 0.16 on the oracle), so the check above does
  depend on the random term being random.
"""
import numpy as np
import pytest

from helpers import make_gpu
from tfg import abi
from tfg.configs import PotSpec, Workload, cells_for, in_box

pytestmark = pytest.mark.gpu


def dpd_box(n, density, flags=0, seed=3):
    """n DPD particles uniform in a periodic cube at the given number density, Maxwell
    velocities at kT = 1 with the mean removed; the droplet workload's DPD parameters."""
    side = float((n / density) ** (1.0 / 3.0))
    rng = np.random.default_rng(np.random.PCG64(seed))
    x = in_box(rng.uniform(0.0, side, (n, 3)), side)
    v = rng.normal(0.0, 1.0, (n, 3))
    v -= v.mean(axis=0)
    c = cells_for(side, 1.0)
    w = Workload(name="dpd_box", origin=(0.0, 0.0, 0.0), dim=(side,) * 3, cells=(c, c, c), cutoff=1.0, dt=0.01,
                 steps=600, x=x, type=np.zeros(n, np.int32), v=v.astype(np.float32),
                 radius=np.ones(n, np.float32), imass=np.ones(n, np.float32), max_type=1,
                 dynamics=[abi.NEWTONIAN], mass=[1.0], seed=77, flags=flags)
    w.pots[(0, 0)] = PotSpec("dpd", dict(alpha=10.0, gamma=4.5, sigma=3.0, cutoff=1.0, shifted=False))
    return w


def _run(w, steps=600, every=10):
    g = make_gpu(w)
    temps, var = [], []
    for _ in range(steps // every):
        g.step(every)
        v = g.download()["v"].astype(np.float64)
        temps.append(float((v ** 2).mean()))
        var.append(v.var(axis=0))
    return g, np.array(temps), np.array(var)


@pytest.mark.parametrize("density", [3.0, 6.9])
def test_dpd_noise_on_equilibrates_at_kt_one(density):
    w = dpd_box(20000, density)
    g, temps, var = _run(w)
    half = len(temps) // 2
    kt = temps[half:].mean()
    print("DPD thermostat, density %.1f: kT = %.4f (std over samples %.4f), component variances %s"
          % (density, kt, temps[half:].std(), np.round(var[half:].mean(axis=0), 4)))
    assert abs(kt - 1.0) < 0.04, kt
    assert np.all(np.abs(var[half:].mean(axis=0) - 1.0) < 0.04)
    v = g.download()["v"].astype(np.float64)
    assert np.all(np.abs(v.mean(axis=0)) < 5e-3)
    kurt = (v ** 4).mean(axis=0) / (v ** 2).mean(axis=0) ** 2
    assert np.all(np.abs(kurt - 3.0) < 0.1), kurt


def test_dpd_reference_constant_term_is_not_a_thermostat():
    w = dpd_box(20000, 3.0, flags=abi.ENGINE_DPD_REFERENCE_RANDOM)
    _, temps, _ = _run(w, steps=300)
    assert temps[-5:].mean() < 0.5, temps[-5:]
