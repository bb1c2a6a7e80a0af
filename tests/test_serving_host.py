"""CPU checks of the serving loop's host logic (gbfv.serving): admission in
arrival order within the slot count and the HBM budget, requests arriving
while others run joining at the next round, a request that cannot fit an
empty server reported, lanes routing by size with one host thread each, and
the latency summary.  A fake server with the loop's interface (try_admit,
running, step, collect) and a fake clock stand in for the device."""
import threading
import types

import numpy as np
import pytest

from gbfv import serving


class FakeClock:
    def __init__(self):
        self.t = 0.0
        self.lock = threading.Lock()

    def __call__(self):
        with self.lock:
            return self.t

    def advance(self, dt):
        with self.lock:
            self.t += dt


class FakeServer:
    """`capacity` slots and a budget in cells; an admitted request runs for
    as many rounds as it has time steps, each round taking `round_s`."""

    def __init__(self, clock, capacity=3, budget=1000, round_s=0.01):
        self.clock, self.capacity, self.budget, self.round_s = clock, capacity, budget, round_s
        self.running, self.left = {}, {}
        self.admitted, self.max_running, self.max_used = [], 0, 0
        self._slot = 0

    def used(self):
        return sum(r.problem.num_cells for r in self.running.values())

    def try_admit(self, req, now):
        if len(self.running) >= self.capacity or self.used() + req.problem.num_cells > self.budget:
            return False
        self._slot += 1
        self.running[self._slot] = req
        self.left[self._slot] = req.steps
        req.admitted, req.slot = now, self._slot
        self.admitted.append(req.rid)
        self.max_running = max(self.max_running, len(self.running))
        self.max_used = max(self.max_used, self.used())
        return True

    def step(self):
        self.clock.advance(self.round_s)
        for s in self.left:
            self.left[s] -= 1

    def collect(self, now, keep_solution=True):
        done = []
        for s in [s for s, k in self.left.items() if k <= 0]:
            req = self.running.pop(s)
            del self.left[s]
            req.status, req.newton = 0, np.full(req.steps, 3, np.int32)
            req.finished = now() if callable(now) else now
            done.append(req)
        return done


def _req(rid, cells, steps=1, arrival=0.0):
    return serving.Request(types.SimpleNamespace(num_cells=cells), steps=steps, arrival=arrival, rid=rid)


@pytest.fixture
def clock(monkeypatch):
    c = FakeClock()
    monkeypatch.setattr(serving.time, "sleep", lambda s: c.advance(max(s, 1e-6)))
    return c


def test_admission_in_arrival_order_within_slots_and_budget(clock):
    srv = FakeServer(clock, capacity=3, budget=1000)
    reqs = [_req(i, 200 + 50 * (i % 3), steps=1 + i % 4) for i in range(12)]
    serving.serve(srv, reqs, clock=clock)
    assert srv.admitted == list(range(12))
    assert srv.max_running <= 3 and srv.max_used <= 1000
    assert all(r.status == 0 and r.finished >= r.admitted >= r.arrival for r in reqs)


def test_requests_are_not_admitted_before_they_arrive(clock):
    srv = FakeServer(clock, capacity=8)
    reqs = [_req(0, 100, steps=2, arrival=0.0), _req(1, 100, arrival=0.5), _req(2, 100, arrival=1.25)]
    serving.serve(srv, reqs, clock=clock)
    for r in reqs:
        assert r.admitted >= r.arrival
        assert r.admitted - r.arrival < 0.02      # at the next round or poll
    assert srv.admitted == [0, 1, 2]


def test_a_request_arriving_while_others_run_joins_the_next_round(clock):
    srv = FakeServer(clock, capacity=4, round_s=0.01)
    long_run = _req(0, 100, steps=50)
    short = _req(1, 100, steps=2, arrival=0.105)
    serving.serve(srv, [long_run, short], clock=clock)
    assert long_run.admitted == 0.0
    assert short.admitted < long_run.finished            # did not wait for the long request
    assert short.finished < long_run.finished
    assert short.admitted - short.arrival <= 0.01 + 1e-12


def test_head_of_line_waits_for_room_then_runs(clock):
    srv = FakeServer(clock, capacity=4, budget=1000)
    big_first = [_req(0, 700, steps=5), _req(1, 600, steps=1), _req(2, 100, steps=1)]
    serving.serve(srv, big_first, clock=clock)
    # arrival order is kept: request 1 waits for the budget request 0 holds,
    # and request 2 waits behind it
    assert srv.admitted == [0, 1, 2]
    assert big_first[1].admitted >= big_first[0].finished


def test_a_request_larger_than_an_empty_server_is_reported(clock):
    srv = FakeServer(clock, capacity=2, budget=500)
    with pytest.raises(RuntimeError, match="does not fit"):
        serving.serve(srv, [_req(0, 100), _req(1, 900)], clock=clock)


def test_lanes_route_by_size_and_run_side_by_side(clock):
    small, large = FakeServer(clock, capacity=4, budget=10 ** 6), FakeServer(clock, capacity=2, budget=10 ** 7)
    laned = object.__new__(serving.LanedServer)
    laned.lanes = [(1000, small), (10 ** 6, large)]
    reqs = [_req(i, 500 if i % 3 else 50000, steps=1 + i % 2, arrival=0.01 * i) for i in range(9)]
    serving.serve_laned(laned, reqs, clock=clock)
    assert sorted(small.admitted) == [i for i in range(9) if i % 3]
    assert sorted(large.admitted) == [i for i in range(9) if not i % 3]
    assert all(r.status == 0 for r in reqs)
    with pytest.raises(ValueError):
        laned.lane_of(types.SimpleNamespace(num_cells=10 ** 6 + 1))


def test_a_failing_lane_is_reported_after_the_others_finish(clock):
    ok, tight = FakeServer(clock, capacity=2, budget=10 ** 6), FakeServer(clock, capacity=2, budget=10)
    laned = object.__new__(serving.LanedServer)
    laned.lanes = [(1000, ok), (10 ** 6, tight)]
    reqs = [_req(0, 500), _req(1, 5000), _req(2, 600, steps=3)]
    with pytest.raises(RuntimeError):
        serving.serve_laned(laned, reqs, clock=clock)
    assert reqs[0].status == 0 and reqs[2].status == 0       # the other lane still ran to the end


def test_latency_summary():
    reqs = []
    for i, (arr, fin, n) in enumerate([(0.0, 1.0, 3), (0.5, 2.5, 4), (1.0, 2.0, 2)]):
        r = _req(i, 1000, steps=1, arrival=arr)
        r.finished, r.newton, r.status = fin, np.array([n]), 0 if i < 2 else 5
        reqs.append(r)
    s = serving.latency_summary(reqs)
    assert s["p50_ms"] == pytest.approx(1000.0) and s["mean_ms"] == pytest.approx(4000.0 / 3)
    assert s["requests"] == 3 and s["throughput_rps"] == pytest.approx(3 / 2.5)
    assert s["cell_newton_its_per_s"] == pytest.approx(9000 / 2.5) and s["failed"] == 1
