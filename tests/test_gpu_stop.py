"""Per-simulation stops (tfg_batch_set_stop) on the GPU.

A batch member told to stop at clock k is left exactly as it is by every later step of the
batch: positions, velocities, cells, species and flux state, its clock, and the totals of
its last step.  The other members are not affected by it, and a stopped member whose stop
is raised continues as if it had not paused.  Checked bit for bit with the deterministic
pair pass (the same kernels, run twice, agree bit for bit), for cell sorting with random
forces, DPD droplets with Fickian flux (flux substeps, species), and a Verlet-mode
Lennard-Jones fluid (rebuild schedule kept across the pause); and, with the tiled pair
kernel, the frozen state itself."""
import numpy as np
import pytest

from tfg import configs
from tfg.engine import Batch, setup_model

pytestmark = pytest.mark.gpu

KEYS = ("xrel", "v", "cell", "species", "q")


def _bits(a):
    a = np.asarray(a)
    return np.ascontiguousarray(a).view(np.uint32) if a.dtype == np.float32 else a


def _same(a, b, what):
    for k in KEYS:
        if k in a and a[k] is not None and np.size(a[k]):
            assert np.array_equal(_bits(a[k]), _bits(b[k])), "%s: %s differs" % (what, k)


def _batch(ws, deterministic=True):
    b = Batch(ws[0].max_type, ws[0].nr_species)
    sims = []
    for w in ws:
        s = b.add_sim(w.desc())
        b._keep.extend(setup_model(s, w))
        sims.append(s)
    b.set_deterministic(deterministic)
    return b, sims


def _members(kind):
    if kind == "cell_sorting":
        return [configs.cell_sorting(n=600, side=11.0, seed=61, random_force=(0.0, 0.1, 1)),
                configs.cell_sorting(n=2500, side=17.0, depth_ab=0.4, seed=62, random_force=(0.0, 0.1, 1)),
                configs.cell_sorting(n=1200, side=13.5, seed=63)]
    if kind == "dpd_flux":
        return [configs.dpd_droplets(n=4000, side=14.0, radius=4.0, seed=64),
                configs.dpd_droplets(n=6000, side=16.0, radius=5.0, seed=65)]
    return [configs.verlet(configs.lj_fluid(n=3000, density=0.8, seed=66), skin=0.3),
            configs.verlet(configs.lj_fluid(n=2000, density=0.8, seed=67), skin=0.3)]


@pytest.mark.parametrize("kind", ["cell_sorting", "dpd_flux", "verlet"])
def test_stop_freezes_one_member_and_resumes(kind):
    k_stop, k_total = 4, 10
    # reference: the same batch, nobody stopped
    ref, rs = _batch(_members(kind))
    ref.step(k_stop)
    at_stop = rs[1].download()
    red_at_stop = rs[1].reductions()
    ref.step(k_total - k_stop)
    ref_end = [s.download() for s in rs]

    b, ss = _batch(_members(kind))
    ss[1].set_stop(k_stop)
    b.step(k_total)
    frozen = ss[1].download()
    _same(frozen, at_stop, "stopped member")
    r = ss[1].reductions()
    assert r.steps == k_stop
    assert abs(r.epot - red_at_stop.epot) <= 1e-12 * max(1.0, abs(red_at_stop.epot))
    assert abs(r.kinetic - red_at_stop.kinetic) <= 1e-12 * max(1.0, abs(red_at_stop.kinetic))
    for i in [j for j in range(len(ss)) if j != 1]:
        _same(ss[i].download(), ref_end[i], "running member %d" % i)
        assert ss[i].reductions().steps == k_total

    # raise the stop: the member continues from clock 4 to clock 10 as if it had not paused
    ss[1].set_stop(-1)
    b.step(k_total - k_stop)
    _same(ss[1].download(), ref_end[1], "resumed member")
    assert ss[1].reductions().steps == k_total


def test_stop_freezes_state_with_the_tiled_kernel():
    ws = _members("cell_sorting")
    b, ss = _batch(ws, deterministic=False)
    ss[0].set_stop(3)
    ss[2].set_stop(0)   # never advances: laid out by the first step, then left alone
    b.step(1)
    start = ss[2].download()
    b.step(2)
    a = ss[0].download()
    b.step(7)
    _same(ss[0].download(), a, "member stopped at 3")
    _same(ss[2].download(), start, "member stopped at 0")
    assert [s.reductions().steps for s in ss] == [3, 10, 0]
    # a member added while the others are stopped joins a re-laid-out arena; the stopped
    # ones stay frozen through the re-layout
    extra = configs.cell_sorting(n=800, side=12.0, seed=68)
    s3 = b.add_sim(extra.desc())
    b._keep.extend(setup_model(s3, extra))
    b.step(2)
    _same(ss[0].download(), a, "member stopped at 3, after a re-layout")
    assert s3.reductions().steps == 2 and ss[1].reductions().steps == 12
