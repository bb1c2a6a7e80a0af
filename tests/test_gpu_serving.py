"""GPU checks of the serving path (gbfv_serve_*, gbfv.serving): requests are
admitted into slots as slots and memory free up, run together with the
requests already on the GPU (continuous batching), and each result is the
same as the same request solved alone (bit-identical state, same Newton and
linear iteration counts)."""
import numpy as np
import pytest

from gbfv import Context, capi, problems
from gbfv.serving import Request, Server, latency_summary, serve

pytestmark = pytest.mark.gpu

CLUSTER = 2


def _prm():
    return capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                               inner_tolerance=1e-5)


def _alone(prob, prm, steps, dt):
    ctx = Context(prob, prm)
    ctx.set_solver_config(capi.PREC_MIXED, 1, CLUSTER)
    st, _, sn, sl, _ = ctx.time_integration(steps, dt, fixed_dt=True)
    out = ctx.solution()
    ctx.close()
    return st, sn, sl, out


def test_requests_join_while_others_run(built):
    prm = _prm()
    probs = [problems.blackoil(10, 9, 3, seed=11), problems.blackoil(14, 12, 4, seed=12),
             problems.blackoil(8, 8, 3, seed=13), problems.blackoil(12, 7, 5, seed=14),
             problems.blackoil(9, 11, 4, seed=15)]
    srv = Server(capi.MODEL_BLACKOIL_3P, prm, capacity=2, cluster_size=CLUSTER, max_cells=4096)
    reqs = [Request(p, steps=2, dt=86400.0, rid=i) for i, p in enumerate(probs)]
    # two slots: the first two start; the others are admitted as slots free up,
    # while the remaining request is still iterating
    waiting = list(reqs)
    overlapped = False
    done = []
    now = 0.0
    while len(done) < len(reqs):
        while waiting and srv.try_admit(waiting[0], now):
            waiting.pop(0)
        running_before = set(srv.running)
        srv.step()
        now += 1.0
        finished = srv.collect(now, keep_solution=True)
        done += finished
        if finished and waiting and len(running_before) == 2:
            overlapped = True
    assert overlapped
    srv.close()
    for req in reqs:
        assert req.status == 0
        st, sn, sl, (x, m) = _alone(req.problem, prm, 2, 86400.0)
        assert st == 0
        assert np.array_equal(req.solution[0], x) and np.array_equal(req.solution[1], m), req.rid


def test_admission_by_footprint(built):
    prm = _prm()
    p = problems.blackoil(10, 10, 3)
    srv = Server(capi.MODEL_BLACKOIL_3P, prm, capacity=8, cluster_size=CLUSTER, max_cells=4096)
    fp = srv.footprint(p)
    assert fp > 300 * 2000
    srv.budget = int(2.5 * fp)          # room for two systems
    reqs = [Request(p, steps=1, rid=i) for i in range(3)]
    assert srv.try_admit(reqs[0], 0.0) and srv.try_admit(reqs[1], 0.0)
    assert not srv.try_admit(reqs[2], 0.0)
    while srv.running:
        srv.step()
        srv.collect(1.0)
    assert srv.used() == 0
    assert srv.try_admit(reqs[2], 2.0)
    srv.close()


def test_served_trace_latencies(built):
    prm = _prm()
    probs = [problems.blackoil(10, 9, 3, seed=21 + i) for i in range(6)]
    rng = np.random.default_rng(5)
    t = np.cumsum(rng.exponential(1 / 200.0, len(probs)))
    reqs = [Request(p, steps=1, arrival=float(a), rid=i) for i, (p, a) in enumerate(zip(probs, t))]
    srv = Server(capi.MODEL_BLACKOIL_3P, prm, capacity=4, cluster_size=CLUSTER, max_cells=4096)
    serve(srv, reqs)
    srv.close()
    s = latency_summary(reqs)
    assert s["requests"] == 6 and s["failed"] == 0
    assert 0 < s["p50_ms"] <= s["p99_ms"]
    assert all(r.admitted >= r.arrival for r in reqs)


def test_laned_server_results_equal_alone(built):
    from gbfv.serving import LanedServer, serve_laned
    prm = _prm()
    probs = [problems.blackoil(10, 9, 3, seed=31), problems.blackoil(16, 14, 5, seed=32),
             problems.blackoil(8, 8, 3, seed=33), problems.blackoil(15, 15, 4, seed=34)]
    laned = LanedServer(capi.MODEL_BLACKOIL_3P, prm, lanes=((400, 2, CLUSTER), (4096, 2, CLUSTER)))
    assert [laned.lane_of(p) for p in probs] == [0, 1, 0, 1]
    reqs = [Request(p, steps=1, arrival=0.001 * i, rid=i) for i, p in enumerate(probs)]
    serve_laned(laned, reqs)
    laned.close()
    for req in reqs:
        assert req.status == 0
        st, sn, sl, (x, m) = _alone(req.problem, prm, 1, 86400.0)
        assert np.array_equal(req.solution[0], x) and np.array_equal(req.solution[1], m), req.rid
