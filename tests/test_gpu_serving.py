"""Served stream: requests admitted while others run on the GPU give the same result as
the same simulation run alone (positions within 1e-3, species within 1e-4, same step
count), and their work overlaps in the arena."""
import numpy as np
import pytest

from helpers import make_gpu
from tfg import configs
from tfg.serving import Request, Server, summarize

pytestmark = pytest.mark.gpu


def _requests():
    specs = [(0, 0.000, configs.cell_sorting(n=400, side=10.0, seed=31), 17),
             (1, 0.000, configs.cell_sorting(n=2200, side=16.0, depth_ab=1.3, seed=32), 40),
             (2, 0.002, configs.dpd_droplets(n=1500, side=10.0, radius=3.0, seed=33), 23),
             (3, 0.004, configs.cell_sorting(n=1200, side=13.5, depth_ab=0.2, seed=34,
                                             random_force=(0.0, 0.1, 1)), 9),
             (4, 0.006, configs.dpd_droplets(n=900, side=9.0, radius=2.5, seed=35), 31),
             (5, 0.010, configs.cell_sorting(n=3100, side=18.4, seed=36), 12),
             (6, 0.012, configs.cell_sorting(n=700, side=11.2, seed=37), 26)]
    return [Request(rid, t, w, steps) for rid, t, w, steps in specs]


def test_served_results_match_alone():
    reqs = _requests()
    srv = Server(max_particles=5000, quantum=8)
    done = srv.run(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    assert srv.max_concurrent >= 2
    for r in done:
        w = r.workload
        g = make_gpu(w)
        g.step(r.steps)
        a, b = r.result, g.download()
        side = np.array(w.dim, np.float32)
        d = a["x"] - b["x"]
        d -= side * np.round(d / side)
        assert np.max(np.abs(d)) < 1e-3, "request %d: max position deviation %.3g" % (r.rid, np.max(np.abs(d)))
        if w.nr_species:
            assert np.max(np.abs(a["species"] - b["species"])) < 1e-4
        assert r.reductions.steps == r.steps
        assert r.t_admit >= r.t_arrival and r.t_done >= r.t_admit
    s = summarize(done)
    assert s["p99_latency_s"] >= s["p50_latency_s"] > 0
