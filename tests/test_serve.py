"""Serving-loop host logic with a fake backend (CPU only): admission by the
HBM budget, SGS-phase alignment of admissions, slot reuse, chunk release,
latency statistics."""
import itertools

from lesgo_gb300.serve import Request, Server, poisson_requests


class FakeHandle:
    def __init__(self, grid, cap):
        self.grid, self.cap, self.members, self.steps = grid, cap, set(), 0
        self.ids = itertools.count()
        self.adm = {}
        self.closed = False


class FakeBackend:
    def __init__(self):
        self.handles = []
        self.admit_steps = []

    def slot_bytes(self, grid):
        nx, ny, nz = grid
        return nx * ny * nz * 100

    def create(self, grid, cap):
        h = FakeHandle(grid, cap)
        self.handles.append(h)
        return h

    def add(self, h, req):
        assert len(h.members) < h.cap
        # steps every current member has done since its admission
        self.admit_steps.extend(h.steps - h.adm[m] for m in h.members)
        i = next(h.ids)
        h.members.add(i)
        h.adm[i] = h.steps
        return i

    def step(self, h):
        h.steps += 1

    def sync(self, h):
        pass

    def collect(self, h, iid, req):
        return {"steps_seen": h.steps}

    def remove(self, h, iid):
        h.members.remove(iid)

    def close(self, h):
        h.closed = True


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-3
        return self.t


def test_all_requests_complete_within_budget():
    be = FakeBackend()
    reqs = poisson_requests(40, rate=200.0, grids=[(16, 16, 16), (32, 32, 16)], steps_range=(3, 12), seed=1)
    budget = 2 * 8 * 32 * 32 * 16 * 100 + 8 * 16 * 16 * 16 * 100      # room for three chunks at most
    srv = Server(be, budget_bytes=budget, chunk_slots=8, cs_count=5, clock=Clock())
    rep = srv.run(reqs, idle_sleep=0)
    assert rep["requests"] == 40
    assert all(r.finished >= r.admitted >= r.arrival for r in srv.done)
    assert rep["p99_s"] >= rep["p50_s"] > 0
    assert rep["point_steps"] == sum(r.points * r.steps for r in reqs)
    assert srv.allocated == 0 and all(h.closed for h in be.handles)


def test_budget_is_never_exceeded_and_requests_wait():
    be = FakeBackend()
    reqs = [Request(i, (32, 32, 16), 1e-4, i, steps=7, arrival=0.0) for i in range(20)]
    one_chunk = 4 * 32 * 32 * 16 * 100
    peak = []

    class Probe(Server):
        def _tick(self):
            peak.append(self.allocated)
            super()._tick()

    srv = Probe(be, budget_bytes=one_chunk, chunk_slots=4, cs_count=5, clock=Clock())
    srv.run(reqs, idle_sleep=0)
    assert max(peak) <= one_chunk
    assert len(srv.done) == 20
    assert len(be.handles) >= 1


def test_admissions_align_with_the_sgs_phase():
    be = FakeBackend()
    reqs = [Request(i, (16, 16, 16), 1e-4, i, steps=3 + i % 4, arrival=0.002 * i) for i in range(30)]
    srv = Server(be, budget_bytes=1e12, chunk_slots=6, cs_count=5, clock=Clock())
    srv.run(reqs, idle_sleep=0)
    assert be.admit_steps and all(s % 5 == 0 for s in be.admit_steps)
