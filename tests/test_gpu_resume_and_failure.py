"""Checkpoint/resume and per-simulation failure on the GPU.

Resume: a run saved at step k (cells, cell-relative positions, velocities, species, the
flux increments particles carry into the next step, and the engine clock that keys every
random stream) and reloaded into a fresh engine (tfg_load_particles_binned +
tfg_batch_resume) continues to step 2k bit-identically to the uninterrupted run: positions,
velocities, cells and species, for the cell-sorting configuration (4,000 particles) and the
DPD droplets with Fickian flux (100,000 particles, noise on).  Both runs use the
deterministic pair pass (tfg_set_deterministic: per-particle accumulation in a fixed order,
no atomics), so two runs can agree bit for bit at all.  The reference restores a saved
Universe through FIO (tfSimulator.cpp:940-1020).

Failure: a non-finite external force planted in one simulation's host arrays makes its
positions non-finite at the first step.  Only that simulation reports TFG_E_NAN
(tfg_batch_sim_status; the reference flags the particle, toofast_error,
tf_engine_advance.cpp:72-85, 204-206); the step call reports the error, the other members
keep their status and, after the failed one is removed, still equal their alone runs.  The
served path retires the failed request with that status while the others finish and equal
their alone runs.  Nothing is injected on the device: the fault is in the host input."""
import numpy as np
import pytest

from helpers import make_gpu
from tfg import abi, configs
from tfg.engine import Batch, Engine, TfgError, setup_model
from tfg.serving import Request, Server

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", ["cell_sorting", "dpd_droplets"])
def test_resume_continues_bit_identically(name):
    w = configs.cell_sorting() if name == "cell_sorting" else configs.dpd_droplets()
    k = 10
    ref = make_gpu(w)
    ref.set_deterministic(True)
    ref.step(2 * k)
    a = ref.download()

    first = make_gpu(w)
    first.set_deterministic(True)
    first.step(k)
    saved = first.download()
    del first
    e = Engine(w.desc())
    e._keep = setup_model(e, w)   # the model; its particles are replaced below
    e.set_deterministic(True)
    e.load_binned(saved["cell"], saved["xrel"], v=saved["v"], type=w.type, radius=w.radius, imass=w.imass,
                  species=saved["species"] if w.nr_species else None)
    e.resume(k, q=saved["q"] if w.nr_species else None)
    e.step(k)
    b = e.download()
    assert e.reductions().steps == 2 * k
    for key in ("xrel", "v"):
        assert np.array_equal(_bits(a[key]), _bits(b[key])), key
    assert np.array_equal(a["cell"], b["cell"])
    if w.nr_species:
        assert np.array_equal(_bits(a["species"]), _bits(b["species"]))


def _members():
    return [configs.cell_sorting(n=300, side=10.0, seed=11),
            configs.cell_sorting(n=2500, side=17.0, depth_ab=0.4, seed=12),
            configs.cell_sorting(n=900, side=12.5, depth_ab=1.7, seed=13)]


def _poison(w):
    f = np.zeros((w.n, 3), np.float32)
    f[5, 0] = np.nan
    w.force_i = f
    return w


def test_failed_simulation_is_isolated_in_a_batch():
    ws = _members()
    ws[1] = _poison(ws[1])
    b = Batch(ws[0].max_type, ws[0].nr_species)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    with pytest.raises(TfgError) as ei:
        b.step(3)
    assert ei.value.code == abi.TFG_E_NAN
    assert [s.status() for s in sims] == [0, abi.TFG_E_NAN, 0]
    b.remove_sim(sims[1])
    b.step(4)
    for s, w in ((sims[0], ws[0]), (sims[2], ws[2])):
        g = make_gpu(w)
        g.step(7)
        x, r = s.download()["x"], g.download()["x"]
        side = np.array(w.dim, np.float32)
        d = x - r
        d -= side * np.round(d / side)
        assert np.max(np.abs(d)) < 1e-3
        assert s.status() == 0


def test_served_failure_is_retired_alone():
    ws = _members()
    ws[2] = _poison(ws[2])
    reqs = [Request(i, 0.0005 * i, w, 12) for i, w in enumerate(ws)]
    srv = Server(max_particles=10 ** 7, quantum=4)
    done = {r.rid: r for r in srv.run(reqs)}
    assert done[2].status == abi.TFG_E_NAN and done[2].result is None
    for rid in (0, 1):
        r = done[rid]
        assert r.status == 0
        g = make_gpu(r.workload)
        g.step(r.steps)
        side = np.array(r.workload.dim, np.float32)
        d = r.result["x"] - g.download()["x"]
        d -= side * np.round(d / side)
        assert np.max(np.abs(d)) < 1e-3
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 2
