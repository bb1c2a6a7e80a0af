"""Request loop over the serving C ABI (gbfv_serve_*): continuous batching of
time-step solves.

Requests arrive over time.  A request is admitted into a free slot of the
server as soon as a slot is free and its estimated device footprint fits the
HBM budget; every server step runs one Newton round for all running
requests on the device at once (one batched launch per phase), so requests
that arrive while others are running join at the next round and their work
overlaps.  A finished request's state is read back and its slot released.
"""
import collections
import ctypes as C
import time

import numpy as np

from . import Context, capi

_d = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
_i = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))   # noqa: E731


class Request:
    """One solve: a problem, its initial state, its time steps."""

    def __init__(self, problem, steps=1, dt=86400.0, arrival=0.0, rid=0, fixed_dt=True):
        self.problem = problem
        self.steps = steps
        self.dt = dt
        self.arrival = arrival
        self.rid = rid
        self.fixed_dt = fixed_dt
        self.admitted = None
        self.finished = None
        self.status = None
        self.solution = None
        self.slot = None
        self.newton = None

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


class Server:
    """A continuous-batching server of one model on one GPU."""

    def __init__(self, model, params, capacity=32, hbm_budget=None, cluster_size=8, max_cells=1 << 21):
        self.lib = capi.load()
        self.params = params
        st = C.c_int()
        self.h = self.lib.gbfv_serve_create(capacity, model, C.byref(params), cluster_size, max_cells, C.byref(st))
        if not self.h:
            capi.check(st.value, "gbfv_serve_create")
        self.capacity = capacity
        if hbm_budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(0.8 * free)
        self.budget = hbm_budget
        self.running = {}  # slot -> Request
        self._keep = {}
        self.rounds = 0

    def footprint(self, problem):
        dim = 3 if problem.info.get("dim", 3) == 3 else 2
        return int(self.lib.gbfv_footprint_bytes(problem.num_cells, problem.b, dim))

    def used(self):
        return int(self.lib.gbfv_serve_footprint(self.h))

    def try_admit(self, req, now):
        """Admit if a slot is free and the footprint fits; False otherwise."""
        if len(self.running) >= self.capacity:
            return False
        if self.used() + self.footprint(req.problem) > self.budget:
            return False
        p = req.problem
        s = p.struct()
        pv = np.ascontiguousarray(p.init_pv, float)
        m = np.ascontiguousarray(p.init_meaning, np.int32)
        slot = C.c_int()
        capi.check(self.lib.gbfv_serve_admit(self.h, C.byref(s), _d(pv), _i(m), req.steps, req.dt,
                                             int(req.fixed_dt), C.byref(slot)), "gbfv_serve_admit")
        self._keep[slot.value] = (s, pv, m)
        req.slot = slot.value
        req.admitted = now
        self.running[slot.value] = req
        return True

    def step(self):
        n = C.c_int()
        capi.check(self.lib.gbfv_serve_step(self.h, C.byref(n)), "gbfv_serve_step")
        self.rounds += 1
        return n.value

    def collect(self, now, keep_solution=True):
        """Finished requests: read their state back to the host, release
        their slots.  `now` is a time, or a callable giving the time after
        the state is on the host."""
        done = []
        for slot, req in list(self.running.items()):
            state, status = C.c_int(), C.c_int()
            self.lib.gbfv_serve_slot(self.h, slot, C.byref(state), C.byref(status))
            if state.value in (2, 3):
                req.status = status.value
                n, nl = C.c_int(), C.c_int()
                st2 = C.c_int()
                sn = np.zeros(max(1, req.steps), np.int32)
                self.lib.gbfv_batch_system_report(self.h, slot, C.byref(st2), C.byref(n), None, _i(sn), None,
                                                  C.byref(nl))
                req.newton = sn[:n.value].copy()
                if keep_solution:
                    ctx = Context(req.problem, self.params, set_initial=False,
                                  handle=self.lib.gbfv_batch_system(self.h, slot))
                    req.solution = ctx.solution()
                    ctx.h = None
                req.finished = now() if callable(now) else now
                capi.check(self.lib.gbfv_serve_release(self.h, slot), "gbfv_serve_release")
                self._keep.pop(slot, None)
                del self.running[slot]
                done.append(req)
        return done

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbfv_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def serve(server, requests, clock=time.perf_counter, keep_solution=True, t0=None):
    """Run a trace of requests (arrival times in seconds from t0, default
    now) through the server; fills admitted / finished (state on the host) /
    status of each."""
    pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
    queue = collections.deque()
    t0 = clock() if t0 is None else t0
    left = len(pending)
    while left:
        now = clock() - t0
        while pending and pending[0].arrival <= now:
            queue.append(pending.popleft())
        while queue and server.try_admit(queue[0], now):
            queue.popleft()
        if server.running:
            server.step()
            left -= len(server.collect(lambda: clock() - t0, keep_solution))
        elif pending:
            time.sleep(max(0.0, min(0.001, pending[0].arrival - now)))
        elif queue:
            raise RuntimeError("a queued request does not fit the server even when it is empty")
    return requests


class LanedServer:
    """Several servers ("lanes") side by side, each for requests up to its
    size limit, each with its own CUDA stream and host thread.  In one lane
    every round waits for its slowest system, so small requests would wait
    for the million-cell solves of large ones; in their own lane they take
    rounds of their own size while the large ones run beside them.  Each lane
    holds a share of the HBM budget and of the GPU's clusters (its capacity
    times its cluster size in blocks)."""

    def __init__(self, model, params, lanes=((150000, 12, 4), (1 << 21, 4, 16)), hbm_budget=None):
        if hbm_budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(0.8 * free)
        shares = [cap * cl for _, cap, cl in lanes]
        self.lanes = []
        for (max_cells, cap, cl), sh in zip(lanes, shares):
            srv = Server(model, params, capacity=cap, cluster_size=cl, max_cells=max_cells,
                         hbm_budget=int(hbm_budget * sh / sum(shares)))
            self.lanes.append((max_cells, srv))

    def lane_of(self, problem):
        for i, (max_cells, _) in enumerate(self.lanes):
            if problem.num_cells <= max_cells:
                return i
        raise ValueError("request larger than every lane")

    def close(self):
        for _, srv in self.lanes:
            srv.close()


def serve_laned(laned, requests, clock=time.perf_counter, keep_solution=True):
    """Run a trace through a LanedServer: one host thread per lane, a common
    time origin."""
    import threading
    parts = [[] for _ in laned.lanes]
    for r in requests:
        parts[laned.lane_of(r.problem)].append(r)
    t0 = clock()
    errors = []

    def run(i):
        try:
            serve(laned.lanes[i][1], parts[i], clock, keep_solution, t0)
        except Exception as e:  # reported after the other lanes finish
            errors.append(e)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(parts)) if parts[i]]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return requests


def serve_one_at_a_time(requests, params, clock=time.perf_counter):
    """Baseline: each request alone through a single context, in arrival
    order (queueing included in its latency)."""
    t0 = clock()
    for req in sorted(requests, key=lambda r: r.arrival):
        now = clock() - t0
        if req.arrival > now:
            time.sleep(req.arrival - now)
        req.admitted = clock() - t0
        ctx = Context(req.problem, params)
        st, _, sn, _, _ = ctx.time_integration(req.steps, req.dt, fixed_dt=req.fixed_dt)
        req.solution = ctx.solution()
        req.status = st
        req.newton = sn
        req.finished = clock() - t0
        ctx.close()
    return requests


def latency_summary(requests):
    lat = np.array([r.latency for r in requests if r.latency is not None])
    span = max(r.finished for r in requests) - min(r.arrival for r in requests)
    cits = sum(int(np.sum(r.newton)) * r.problem.num_cells for r in requests if r.newton is not None)
    arr = sorted(r.arrival for r in requests)
    offered = (len(arr) - 1) / (arr[-1] - arr[0]) if len(arr) > 1 and arr[-1] > arr[0] else None
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "max_ms": float(lat.max() * 1e3), "mean_ms": float(lat.mean() * 1e3), "requests": len(lat),
            "offered_rps": offered, "throughput_rps": len(lat) / span,
            "cell_newton_its_per_s": cits / span, "failed": int(sum(1 for r in requests if r.status))}
