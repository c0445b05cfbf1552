"""Host logic of the request loop with a stand-in batch (no GPU): least-work-first and
first-come-first-served admission under the particle cap and the byte budget, chunks cut at
the earliest finishing simulation, every request run for exactly its step count."""
import pytest

from tfg import configs
from tfg.serving import Lane, Request, Server, footprint, summarize


class FakeSim:
    def __init__(self, sid, n):
        self.sid = sid
        self.n = n
        self.steps = 0

    def download(self):
        return {"steps": self.steps}

    def reductions(self):
        return {"steps": self.steps}


class FakeBatch:
    """Counts steps per simulation the way the arena advances all live simulations."""

    def __init__(self):
        self.sims = {}
        self.next = 0
        self.log = []
        self._keep = []

    def add_sim(self, desc):
        s = FakeSim(self.next, 0)
        self.sims[self.next] = s
        self.next += 1
        return s

    def remove_sim(self, sim):
        del self.sims[sim.sid]

    def step(self, n, sync=True):
        self.log.append((n, len(self.sims)))
        for s in self.sims.values():
            s.steps += n
        self.polls = 3

    def idle(self):
        # busy for a few polls, so that requests arrive while a chunk is in flight
        self.polls = getattr(self, "polls", 0) - 1
        return self.polls <= 0

    def sync(self):
        pass


class FakeLane(Lane):
    def __init__(self, max_type, nspec):
        super().__init__(max_type, nspec, batch=FakeBatch())

    def admit(self, req):
        from tfg.serving import _Active
        sim = self.batch.add_sim(None)
        sim.n = req.workload.n
        self.active[sim.sid] = _Active(req, sim, [])


def _reqs():
    out = []
    for i, (n, steps, t) in enumerate([(500, 30, 0.0), (900, 7, 0.0005), (300, 64, 0.001), (2000, 15, 0.0015),
                                       (800, 5, 0.002), (1200, 40, 0.0025)]):
        out.append(Request(i, t, configs.cell_sorting(n=n, side=12.0, seed=i), steps))
    return out


def test_every_request_runs_exactly_its_steps():
    lanes = []

    def factory(mt, ns):
        lanes.append(FakeLane(mt, ns))
        return lanes[-1]

    srv = Server(max_particles=2500, quantum=16, lane_factory=factory)
    done = srv.run(_reqs())
    assert len(done) == 6
    for r in done:
        assert r.result["steps"] == r.steps
    # the particle cap held: never more than 2500 particles in flight, except one request alone
    assert srv.max_concurrent >= 2
    for n, live in lanes[0].batch.log:
        assert 1 <= n <= 16
    s = summarize(done)
    assert s["requests"] == 6 and s["p99_latency_s"] >= s["p50_latency_s"]


def test_fifo_admission_and_budget():
    reqs = _reqs()
    budget = 2 * max(footprint(r.workload) for r in reqs)
    srv = Server(max_particles=10 ** 9, budget_bytes=budget, quantum=8, lane_factory=lambda mt, ns: FakeLane(mt, ns),
                 policy="fifo")
    done = srv.run(reqs)
    admits = sorted(done, key=lambda r: (r.t_admit, r.rid))
    assert [r.rid for r in admits] == sorted(r.rid for r in done)   # first come, first served
    assert srv.bytes_in_flight == 0 and srv.particles_in_flight == 0
    big = Request(99, 0.0, configs.cell_sorting(n=500_000, side=100.0, seed=1), 1)
    with pytest.raises(ValueError):
        Server(budget_bytes=1 << 20, lane_factory=lambda mt, ns: FakeLane(mt, ns)).run([big])


def test_least_work_first_among_arrived_requests():
    """With room for one simulation at a time, the requests waiting when a slot frees are
    admitted in order of particles x steps; with "fifo", in arrival order."""
    reqs = [Request(i, 0.0, configs.cell_sorting(n=n, side=12.0, seed=i), steps)
            for i, (n, steps) in enumerate([(800, 20), (900, 30), (300, 5), (600, 4), (700, 40)])]
    srv = Server(max_particles=1000, quantum=64, lane_factory=lambda mt, ns: FakeLane(mt, ns))
    done = srv.run(reqs)
    order = [r.rid for r in sorted(done, key=lambda r: (r.t_admit, r.rid))]
    assert order == sorted(range(5), key=lambda i: reqs[i].workload.n * reqs[i].steps)
    reqs2 = [Request(r.rid, 0.0, r.workload, r.steps) for r in reqs]
    srv = Server(max_particles=1000, quantum=64, lane_factory=lambda mt, ns: FakeLane(mt, ns), policy="fifo")
    done = srv.run(reqs2)
    assert [r.rid for r in sorted(done, key=lambda r: (r.t_admit, r.rid))] == list(range(5))
    for r in done:
        assert r.result["steps"] == r.steps
