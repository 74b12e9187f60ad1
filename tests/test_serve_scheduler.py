"""Serving scheduler on the CPU: admission under the byte budget, LRU
eviction, one solve per system, FIFO dispatch and failures injected among
the request producers, with a stand-in executor that completes each request
after a fixed wall time (no GPU)."""

import threading
import time

import numpy as np
import pytest

from warp_preconditioners_gb300 import serve


class FakeExecutor:
    def __init__(self, slots=2, sizes=None, duration=0.003, fail_rids=()):
        self.slots = slots
        self.sizes = sizes or {}
        self.duration = duration
        self.fail_rids = set(fail_rids)
        self.built, self.released, self.started = [], [], []
        self.in_flight = {}
        self.max_per_key = 0
        self.lock = threading.Lock()

    def estimate(self, key):
        return self.sizes.get(key, 100)

    def build(self, key):
        self.built.append(key)
        return key, self.sizes.get(key, 100)

    def release(self, handle):
        self.released.append(handle)

    def start(self, slot, handle, req, rhs):
        if req.rid in self.fail_rids:
            raise ValueError("planted launch failure")
        self.started.append((time.perf_counter(), slot, req.rid))
        self.in_flight[req.key] = self.in_flight.get(req.key, 0) + 1
        self.max_per_key = max(self.max_per_key, self.in_flight[req.key])
        return [time.perf_counter() + self.duration, req, rhs]

    def poll(self, token):
        return time.perf_counter() >= token[0]

    def finish(self, token):
        req = token[1]
        self.in_flight[req.key] -= 1
        return token[2], [7] * req.k


def reqs(keys, gap=0.0005, k=2):
    return [serve.Request(i, key[0], key[1], k, i * gap, i) for i, key in enumerate(keys)]


def small_rhs(req):
    return np.full((2, req.k), float(req.rid))


def test_stream_is_seeded_and_in_range():
    a = serve.request_stream(200, rate=5.0, seed=0)
    b = serve.request_stream(200, rate=5.0, seed=0)
    assert a == b
    sides = [r.side for r in a]
    assert min(sides) >= round(5e3 ** (1 / 3)) and max(sides) <= round(5e5 ** (1 / 3))
    assert {r.kind for r in a} == set(serve.KINDS)
    assert all(1 <= r.k <= 8 for r in a)
    arr = np.array([r.arrival for r in a])
    assert (np.diff(arr) > 0).all()
    # Poisson arrivals: mean gap ~ 1/rate
    assert abs(np.diff(arr).mean() - 0.2) < 0.05
    assert serve.request_stream(200, rate=5.0, seed=1) != a


def test_rhs_is_seeded_uniform():
    r = serve.Request(0, "laplacian", 5, 3, 0.0, 42)
    x = serve.request_rhs(r)
    assert tuple(x.shape) == (125, 3)
    assert x.abs().max() <= 1.0
    assert (x == serve.request_rhs(r)).all()


def test_all_served_and_fifo_per_system():
    ex = FakeExecutor(slots=3)
    keys = [("laplacian", 10 + (i % 4)) for i in range(24)]
    srv = serve.Server(ex, budget_bytes=10_000)
    out = srv.run(reqs(keys), make_rhs=small_rhs)
    assert all(r.ok for r in out)
    assert all(r.start >= r.arrival - 1e-9 and r.done >= r.start for r in out)
    assert all(r.iterations == [7, 7] for r in out)
    # one solve in flight per system; per system, requests start in arrival order
    assert ex.max_per_key == 1
    order = [rid for _, _, rid in sorted(ex.started)]
    for key in set(keys):
        mine = [rid for rid in order if keys[rid] == key]
        assert mine == sorted(mine)
    assert ex.built.count(("laplacian", 10)) == 1  # resident after first use


def test_budget_evicts_least_recently_used():
    ex = FakeExecutor(slots=1, sizes={("laplacian", s): 100 for s in range(5)})
    srv = serve.Server(ex, budget_bytes=250)
    keys = [("laplacian", 0), ("laplacian", 1), ("laplacian", 0), ("laplacian", 2)]
    out = srv.run(reqs(keys, gap=0.01), make_rhs=small_rhs)
    assert all(r.ok for r in out)
    assert ex.released == [("laplacian", 1)]  # 0 was used more recently
    assert srv.peak <= 250 and srv.used <= 250
    assert srv.stats["evictions"] == 1


def test_over_budget_system_is_rejected():
    ex = FakeExecutor(slots=2, sizes={("biharmonic", 70): 10_000})
    srv = serve.Server(ex, budget_bytes=1_000)
    keys = [("laplacian", 3), ("biharmonic", 70), ("laplacian", 4)]
    out = srv.run(reqs(keys), make_rhs=small_rhs)
    assert out[0].ok and out[2].ok
    assert not out[1].ok and "budget" in out[1].error
    assert srv.stats["rejected"] == 1
    assert ("biharmonic", 70) not in ex.built


def test_waits_for_room_while_systems_are_busy():
    # Two systems of 100 bytes under a 150-byte budget: the second waits
    # until the first is idle and evictable.
    ex = FakeExecutor(slots=2, sizes={("laplacian", 1): 100, ("laplacian", 2): 100},
                      duration=0.02)
    srv = serve.Server(ex, budget_bytes=150)
    out = srv.run(reqs([("laplacian", 1), ("laplacian", 2)], gap=0.0), make_rhs=small_rhs)
    assert all(r.ok for r in out)
    assert out[1].start >= out[0].done - 1e-3
    assert srv.peak <= 150


def test_producer_failure_is_reported_per_request():
    def make(req):
        if req.rid == 3:
            raise IOError("planted read failure")
        return small_rhs(req)

    out = serve.Server(FakeExecutor(), budget_bytes=10_000).run(
        reqs([("laplacian", 5)] * 8), make_rhs=make)
    assert not out[3].ok and "producer failed" in out[3].error and "planted" in out[3].error
    assert all(r.ok for i, r in enumerate(out) if i != 3)


@pytest.mark.filterwarnings("ignore::pytest.PytestUnhandledThreadExceptionWarning")
def test_stopped_producer_does_not_hang_the_server():
    def make(req):
        if req.rid == 4:
            raise SystemExit  # ends the producer thread quietly
        return small_rhs(req)

    box = {}
    t = threading.Thread(target=lambda: box.setdefault(
        "out", serve.Server(FakeExecutor(), budget_bytes=10_000).run(
            reqs([("laplacian", 5)] * 10), make_rhs=make)))
    t.start()
    t.join(timeout=20)
    assert not t.is_alive(), "server hung after its producer stopped"
    out = box["out"]
    assert all(r.ok for r in out[:4])
    assert all(not r.ok and "stopped" in r.error for r in out[4:])


def test_launch_failure_frees_the_slot():
    ex = FakeExecutor(slots=1, fail_rids={1})
    out = serve.Server(ex, budget_bytes=10_000).run(reqs([("laplacian", 5)] * 4),
                                                     make_rhs=small_rhs)
    assert not out[1].ok and "planted launch failure" in out[1].error
    assert out[0].ok and out[2].ok and out[3].ok


def test_summary():
    out = serve.Server(FakeExecutor(), budget_bytes=10_000).run(
        reqs([("laplacian", 5)] * 6, k=3), make_rhs=small_rhs)
    s = serve.summarize(out)
    assert s["completed"] == 6 and s["rhs_solved"] == 18
    assert 0 < s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert s["solves_per_s"] > 0


def test_estimate_bounds_host_sizes():
    host = serve.host_system("laplacian", 6)
    assert host.n == 216 and host.A.shape == (216, 216)
    e8 = serve.estimate_bytes(host, 8)
    assert e8 > serve.estimate_bytes(host, 2) > 0
    with pytest.raises(ValueError):
        serve.host_system("plate", 4)


class MergingExecutor(FakeExecutor):
    """FakeExecutor that also takes several queued requests of one system as
    one solve (start_group / finish_group), like GpuExecutor(merge_rhs=...)."""

    def __init__(self, merge_rhs, **kw):
        super().__init__(**kw)
        self.merge_rhs = merge_rhs
        self.groups = []

    def start_group(self, slot, handle, reqs, rhss):
        assert len(reqs) == len(rhss) > 1
        assert len({r.key for r in reqs}) == 1
        assert sum(r.k for r in reqs) <= self.merge_rhs
        self.groups.append([r.rid for r in reqs])
        self.in_flight[reqs[0].key] = self.in_flight.get(reqs[0].key, 0) + 1
        self.max_per_key = max(self.max_per_key, self.in_flight[reqs[0].key])
        return [time.perf_counter() + self.duration, reqs, rhss]

    def finish_group(self, token):
        reqs, rhss = token[1], token[2]
        self.in_flight[reqs[0].key] -= 1
        return [(rhs, [7] * r.k) for r, rhs in zip(reqs, rhss)]


def test_queued_requests_of_one_system_are_merged():
    key_a, key_b = ("laplacian", 5), ("biharmonic", 4)
    stream = [serve.Request(i, *(key_a if i % 3 else key_b), 2, 0.0, i) for i in range(12)]
    ex = MergingExecutor(merge_rhs=6, slots=1, duration=0.002)
    out = serve.Server(ex).run(stream, make_rhs=small_rhs)
    assert all(r.ok for r in out)
    # every request got its own right-hand sides back, in arrival order
    for req, r in zip(stream, out):
        assert float(r.x[0, 0]) == float(req.rid) and r.iterations == [7, 7]
    assert ex.max_per_key == 1
    merged = [g for g in ex.groups]
    assert merged and all(len(g) <= 3 for g in merged)
    # groups keep arrival order inside a system
    for g in merged:
        assert g == sorted(g)
    # a merge never mixes systems and covers every request exactly once
    started = [rid for _, _, rid in ex.started] + [rid for g in merged for rid in g]
    assert sorted(started) == list(range(12))
