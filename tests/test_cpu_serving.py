"""The native request loop (tissue-forge_gb300/host/tfg_server.cpp) on the CPU.

The server's own code is compiled with a stand-in for the batch C ABI
(tests/fakes/fake_batch.cpp: a simulation is a particle count and a step counter) into a
test library, and driven through the Python client exactly as on the GPU.  Checked here:
every request runs exactly its step count, chunks never exceed the quantum and run whole
(members that finish inside a chunk stop themselves: tfg_batch_set_stop), the particle cap
and the byte budget hold, least-work-first and first-come-first-served admission orders,
and a request whose particles fail is retired with its status while the others finish."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from tfg import abi, configs
from tfg.serving import Request, Server, footprint, summarize

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "fakes", "_build", "libtfg_serverfake.so")


@pytest.fixture(scope="module")
def fake():
    srcs = [os.path.join(ROOT, "tissue-forge_gb300", "host", "tfg_server.cpp"),
            os.path.join(HERE, "fakes", "fake_batch.cpp")]
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or any(os.path.getmtime(s) > os.path.getmtime(OUT) for s in srcs):
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-Wl,-Bsymbolic",
                               "-I" + os.path.join(ROOT, "include"), "-o", OUT] + srcs)
    L = C.CDLL(OUT)
    abi.declare_server_api(L)
    L.tfg_fake_log.argtypes = [C.POINTER(C.c_int)] * 5
    return L


def _log(L):
    v = [C.c_int() for _ in range(5)]
    L.tfg_fake_log(*[C.byref(x) for x in v])
    return dict(zip(("max_chunk", "min_chunk", "max_live", "chunks", "masked"), (x.value for x in v)))


def _reqs():
    out = []
    for i, (n, steps, t) in enumerate([(500, 30, 0.0), (900, 7, 0.0005), (300, 64, 0.001), (2000, 15, 0.0015),
                                       (800, 5, 0.002), (1200, 40, 0.0025)]):
        out.append(Request(i, t, configs.cell_sorting(n=n, side=12.0, seed=i), steps))
    return out


def test_every_request_runs_exactly_its_steps(fake):
    _log(fake)
    srv = Server(max_particles=2500, quantum=16, lib=fake)
    done = srv.run(_reqs())
    assert len(done) == 6
    for r in done:
        assert r.status == 0
        assert np.all(r.result["x"] == r.steps), r.rid   # the stand-in reports its step count
        assert r.reductions.steps == r.steps
        assert r.t_admit >= r.t_arrival and r.t_done >= r.t_admit
    log = _log(fake)
    assert 1 <= log["min_chunk"] and log["max_chunk"] <= 16
    # members finishing inside a chunk were stopped there (masked steps) instead of the
    # chunk being cut for them
    assert log["masked"] > 0 and log["max_chunk"] == 16
    assert srv.max_concurrent >= 2 and log["max_live"] >= 2
    st = srv.stats()
    assert st["completed"] == 6 and st["particles_in_flight"] == 0 and st["bytes_in_flight"] == 0
    s = summarize(done)
    assert s["requests"] == 6 and s["p99_latency_s"] >= s["p50_latency_s"]


def test_particle_cap_holds(fake):
    """With a 1,000-particle cap at most one of these 800-900 particle requests is in flight."""
    reqs = [Request(i, 0.0, configs.cell_sorting(n=800 + 50 * i, side=12.0, seed=i), 6) for i in range(3)]
    _log(fake)
    srv = Server(max_particles=1000, quantum=4, lib=fake)
    done = srv.run(reqs)
    assert all(r.status == 0 for r in done)
    assert _log(fake)["max_live"] == 1 and srv.max_concurrent == 1


def test_fifo_admission_and_budget(fake):
    reqs = _reqs()
    budget = 2 * max(footprint(r.workload) for r in reqs)
    srv = Server(max_particles=10 ** 9, budget_bytes=budget, quantum=8, policy="fifo", lib=fake)
    done = srv.run(reqs)
    admits = sorted(done, key=lambda r: (r.t_admit, r.rid))
    assert [r.rid for r in admits] == sorted(r.rid for r in done)   # first come, first served
    st = srv.stats()
    assert st["bytes_in_flight"] == 0 and st["particles_in_flight"] == 0
    big = Request(99, 0.0, configs.cell_sorting(n=500_000, side=100.0, seed=1), 1)
    with pytest.raises(ValueError):
        Server(budget_bytes=1 << 20, lib=fake).run([big])


def test_least_work_first_among_arrived_requests(fake):
    """With room for one simulation at a time, the requests waiting when a slot frees are
    admitted in order of particles x steps; with "fifo", in arrival order."""
    reqs = [Request(i, 0.0, configs.cell_sorting(n=n, side=12.0, seed=i), steps)
            for i, (n, steps) in enumerate([(800, 20), (900, 30), (300, 5), (600, 4), (700, 40)])]
    srv = Server(max_particles=1000, quantum=64, lib=fake)
    done = srv.run(reqs)
    # the server's own admission times order the admissions exactly (requests admitted in the
    # same turn are mapped onto the client clock through their own submission times)
    order = [r.rid for r in sorted(done, key=lambda r: r.t_admit_server)]
    assert order == sorted(range(5), key=lambda i: reqs[i].workload.n * reqs[i].steps)
    reqs2 = [Request(r.rid, 0.0, r.workload, r.steps) for r in reqs]
    srv = Server(max_particles=1000, quantum=64, policy="fifo", lib=fake)
    done = srv.run(reqs2)
    assert [r.rid for r in sorted(done, key=lambda r: r.t_admit_server)] == list(range(5))
    for r in done:
        assert np.all(r.result["x"] == r.steps)


def test_failed_request_is_retired_alone(fake):
    """A request whose particles fail (a non-finite coordinate, planted in its host arrays)
    comes back with TFG_E_NAN and no result; the others in its batch finish normally."""
    reqs = _reqs()
    w = reqs[3].workload
    w.x = np.array(w.x, np.float32, copy=True)
    w.x[7, 1] = np.nan
    srv = Server(max_particles=10 ** 9, quantum=8, lib=fake)
    done = srv.run(reqs)
    by = {r.rid: r for r in done}
    assert by[3].status == abi.TFG_E_NAN and by[3].result is None
    for rid, r in by.items():
        if rid != 3:
            assert r.status == 0 and np.all(r.result["x"] == r.steps)
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 5
    s = summarize(done)
    assert s["failed"] == 1


def test_lazily_built_requests(fake):
    """Requests built when they arrive (Request(..., None, steps, make=...)) run like the
    others; after submission the client keeps only their shape."""
    built = []

    def make(i, n):
        def f():
            built.append(i)
            return configs.cell_sorting(n=n, side=12.0, seed=i)
        return f

    reqs = [Request(i, 0.0005 * i, None, 5 + i, make=make(i, 400 + 100 * i)) for i in range(4)]
    srv = Server(max_particles=10 ** 9, quantum=4, lib=fake)
    done = srv.run(reqs)
    assert sorted(built) == [0, 1, 2, 3]
    for r in done:
        assert r.status == 0 and np.all(r.result["x"] == r.steps)
        assert r.workload.n == 400 + 100 * r.rid and not hasattr(r.workload, "x")
