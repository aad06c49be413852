"""Serving loop scheduling on CPU: a fake backend with a virtual clock stands
in for the device (no GPU, no C library)."""
import numpy as np
import pytest

from phonomena_gb300 import serve
from phonomena_gb300.crystal import CrystalSpec


class FakeBackend:
    """Instances advance one step per step() call unit; each step costs
    `cost` virtual seconds per million nodes in the mix."""

    def __init__(self, budget, capacity, cost=1e-3):
        self.t = 0.0
        self.cost = cost
        self.budget = budget
        self.capacity = capacity
        self.active = {}   # slot -> [prep, remaining, done]
        self.pool = {}     # key -> count
        self.live = 0      # bytes held (active + pooled)
        self.peak = 0
        self.max_active = 0
        self.steps_log = []
        self.diverging = set()  # requests whose simulation "overflows" after 20 steps

    def clock(self):
        return self.t

    def footprint(self, shape, steps, record_every):
        return int(np.prod(shape)) * 100

    def key(self, p):
        return tuple(p.shape)

    def has_pooled(self, key):
        return self.pool.get(key, 0) > 0

    def evict_one(self, keep=None):
        for k, n in self.pool.items():
            if n and k != keep:
                self.pool[k] -= 1
                b = self.footprint(k, 0, 0)
                self.live -= b
                return b
        return 0

    def admit(self, p):
        k = self.key(p)
        if self.pool.get(k, 0):
            self.pool[k] -= 1
        else:
            self.live += self.footprint(p.shape, 0, 0)
        assert self.live <= self.budget, "memory budget exceeded"
        slot = next(s for s in range(self.capacity) if s not in self.active)
        self.active[slot] = [p, p.req.steps, 0]
        self.max_active = max(self.max_active, len(self.active))
        self.peak = max(self.peak, self.live)
        return slot, p

    def step(self, n):
        nodes = sum(np.prod(a[0].shape) for a in self.active.values() if a[1] > 0)
        self.t += n * self.cost * nodes / 1e6
        self.steps_log.append((n, len(self.active)))
        for a in self.active.values():
            adv = min(n, a[1])
            a[1] -= adv
            a[2] += adv

    def sync(self):
        bad = [s for s, a in self.active.items() if a[0].req.rid in self.diverging and a[2] >= 20]
        return bad

    def remaining(self, slot):
        return self.active[slot][1]

    def finish(self, slot, sim):
        p, rem, done = self.active.pop(slot)
        assert (rem == 0 and done == p.req.steps) or p.req.rid in self.diverging
        k = self.key(p)
        self.pool[k] = self.pool.get(k, 0) + 1
        # the "surface" of a request depends on its own inputs only
        return np.full((p.req.steps // p.req.record_every, 2, 2), p.req.rid * 1000.0 + p.req.steps)


def fake_prepare(req):
    return serve.Prepared(req, req.spec.nodes, {}, None, None, 1e-9, None)


def stream(n, seed=0, rate=50.0):
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for q in range(n):
        t += rng.exponential(1 / rate)
        cells = tuple(int(c) for c in rng.choice([20, 30, 40], size=3))
        steps = int(rng.integers(50, 300))
        out.append(serve.Request(q, CrystalSpec(cells=cells, steps=steps), steps, t))
    return out


def run(reqs, budget, capacity, chunk=60, diverging=()):
    be = FakeBackend(budget, capacity)
    be.diverging = set(diverging)
    srv = serve.Server(be, budget_bytes=budget, capacity=capacity, chunk=chunk, prepare_fn=fake_prepare,
                       clock=be.clock, workers=2)
    res = srv.run(reqs, realtime=False)
    srv.close()
    return be, srv, res


def test_every_request_served_with_its_own_result():
    reqs = stream(40)
    be, srv, res = run(reqs, budget=20 * 41 ** 3 * 100, capacity=6)
    assert sorted(r.rid for r in res) == list(range(40))
    for r in res:
        assert r.surface.shape[0] == r.steps // 10
        assert np.all(r.surface == r.rid * 1000.0 + r.steps)
        assert r.finished >= r.admitted >= 0


def test_budget_and_slots_are_respected():
    reqs = stream(60, seed=1)
    budget = 3 * 41 ** 3 * 100  # about three of the largest at once
    be, srv, res = run(reqs, budget=budget, capacity=4)
    assert len(res) == 60
    assert be.peak <= budget
    assert be.max_active <= 4
    assert srv.stats.peak_bytes <= budget


def test_requests_join_a_running_batch():
    """Continuous batching: a request is admitted while earlier ones are still running."""
    reqs = stream(30, seed=2)
    be, srv, res = run(reqs, budget=10 ** 12, capacity=8)
    by_rid = {r.rid: r for r in res}
    overlaps = sum(1 for a in res for b in res if a.rid < b.rid and b.admitted < by_rid[a.rid].finished)
    assert overlaps > 0
    assert max(n for _, n in be.steps_log) > 1
    # chunk boundaries at each finish: no request overruns its step count
    assert all(r.surface.shape[0] == r.steps // 10 for r in res)


def test_oversized_request_is_rejected_not_stuck():
    reqs = stream(5, seed=3)
    big = serve.Request(99, CrystalSpec(cells=(200, 200, 200), steps=100), 100, 0.01)
    be, srv, res = run(reqs + [big], budget=5 * 41 ** 3 * 100, capacity=4)
    assert srv.stats.rejected == [99]
    assert sorted(r.rid for r in res) == list(range(5))


def test_summary_percentiles():
    reqs = stream(20, seed=4)
    be, srv, res = run(reqs, budget=10 ** 12, capacity=8)
    s = serve.summarize(res)
    lat = sorted(r.latency for r in res)
    assert s["requests"] == 20
    assert s["p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert s["p99_s"] <= lat[-1] + 1e-12 and s["p99_s"] >= s["p95_s"] >= s["p50_s"]
    assert s["gcell_updates_per_s"] > 0


def test_poisson_stream_distribution():
    reqs = serve.poisson_stream(400, rate=10.0, seed=0)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    assert 30 < arr[-1] < 50  # 400 arrivals at 10/s
    steps = np.array([r.steps for r in reqs])
    assert steps.min() >= 500 and steps.max() <= 3000
    large = sum(1 for r in reqs if r.spec.cells == (512, 512, 128))
    assert 5 <= large <= 40
    for r in reqs:
        if r.spec.cells != (512, 512, 128):
            assert r.spec.cells[0] in (64, 96, 128, 160, 192) and r.spec.cells[2] in (32, 48, 64, 96)


def test_failed_request_ends_alone():
    """A simulation with non-finite values ends early with an error; the others finish normally."""
    reqs = stream(12, seed=5)
    be, srv, res = run(reqs, budget=10 ** 12, capacity=4, diverging={3})
    by = {r.rid: r for r in res}
    assert sorted(by) == list(range(12))
    assert by[3].error and by[3].steps < reqs[3].steps
    assert all(r.error is None and r.steps == reqs[r.rid].steps for r in res if r.rid != 3)
    assert serve.summarize(res)["failed"] == 1
