#!/usr/bin/env python
"""Benchmark: cell-Newton-iterations/s of the ECFV/TPFA linearization +
BiCGStab/ILU0 Newton solve on the three-phase black-oil grid
100x100x20 (200k cells, 3x3 blocks), 10 time steps of 1 day.

One bench step = the whole 10-time-step run from the initial state (restored
on the device before each step).  value = sum over time steps of Newton
iterations x cells / device time, for the mixed-precision form (FP64
residual/Jacobian/update/outer residual, FP32 ILU0 + FP32 BiCGStab inside
FP64 iterative refinement, linear tolerance 1e-6 relative).  The plain FP64
form is measured on the same workload and reported beside it.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
For N > 1 (torchrun, one rank per GPU) every rank runs its own replica: the
path has no data-path collective, scaling is weak.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "opm-models_gb300"))

import numpy as np  # noqa: E402

WORKLOADS = {
    "blackoil-100x100x20": dict(nx=100, ny=100, nz=20, steps=10, dt=86400.0),
    "blackoil-100x100x100": dict(nx=100, ny=100, nz=100, steps=10, dt=86400.0),
    "blackoil-50x50x20": dict(nx=50, ny=50, nz=20, steps=10, dt=86400.0),
}
METRIC = "cell-Newton-iters/s (mixed vs plain FP64, same tol); served solve p50/p99 ms"
UNIT = "cell-Newton-iters/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="blackoil-100x100x20", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ensemble", type=int, default=0,
                    help="batched ensemble of this many two-phase realizations (10k-200k cells) instead of "
                         "the single-grid workload")
    ap.add_argument("--serve", action="store_true",
                    help="served stream: Poisson arrivals of single-time-step black-oil solves (20k-1M cells)")
    ap.add_argument("--linearizers", action="store_true",
                    help="linearization only: the AD and the finite-difference local linearizers (forward, "
                         "central) on the workload's initial state, device time per call, and the CPU oracle's")
    ap.add_argument("--profile-case", action="store_true",
                    help="one linearization + one mixed solve of the workload (for ncu captures); "
                         "prints the solve's iterations, launches and algorithmic bytes")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        self.file.close()
        os.unlink(self.file.name)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def build_problem(wl):
    from gbfv import problems
    w = WORKLOADS[wl]
    return problems.blackoil(w["nx"], w["ny"], w["nz"])


def params(precision):
    from gbfv import capi
    # inner FP32 solves to the outer tolerance: fewest total iterations on
    # this workload (1e-5, 3e-6, 1e-6, 5e-7 tried)
    return capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=precision,
                               inner_tolerance=1e-6)


def cpu_sample(prob, iters=2, threads=None):
    """The oracle (the reference algorithm restated on the CPU) on the first
    `iters` Newton iterations of the first time step: OpenMP over elements in
    the linearization, sequential BiCGStab/ILU0 (as the reference)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    orc = O.Oracle(prob, params(0))
    t0 = time.perf_counter()
    for it in range(iters):
        st = orc.linearize(86400.0, it)
        if st:
            raise RuntimeError("oracle linearize failed %d" % st)
        st, _, _ = orc.solve()
        orc.newton_update()
    dt = time.perf_counter() - t0
    orc.close()
    return iters * prob.num_cells / dt, dt, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    prob = build_problem(args.workload)
    for _ in range(args.warmup):
        cpu_sample(prob)
    vals, tot = [], 0.0
    for _ in range(args.steps):
        v, dt, threads = cpu_sample(prob)
        vals.append(v)
        tot += dt
    value = args.steps * 2 * prob.num_cells / tot
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lognormal permeability, uniform porosity)",
        "config": {"workload": args.workload + " black-oil, first 2 Newton iterations of time step 1",
                   "cells": prob.num_cells, "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "2 Newton iterations (linearize + BiCGStab/ILU0 to 1e-6 + update) of "
                                   "time step 1 of the %s workload, per step" % args.workload},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def timed_runs(ctx, w, steps, warmup, flush, torch, ext):
    """Device-time K full runs (restore state on device, 10 time steps)."""
    its = []
    for _ in range(warmup):
        ctx.restore_state()
        st, sdt, sn, sl, tl = ctx.time_integration(w["steps"], w["dt"], fixed_dt=True)
        if st:
            raise RuntimeError("warm-up run failed %d" % st)
    ms_tot, cells_its = 0.0, 0
    launches0 = ctx.lib.gbfv_kernel_launches()
    ctx.reset_kernel_stats()
    for _ in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()  # write a buffer larger than L2 between timed steps
        ctx.restore_state()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        st, sdt, sn, sl, tl = ctx.time_integration(w["steps"], w["dt"], fixed_dt=True)
        e1.record(ext)
        e1.synchronize()
        if st:
            raise RuntimeError("timed run failed %d" % st)
        ms_tot += e0.elapsed_time(e1)
        cells_its += int(sn.sum()) * ctx.N
        its.append((sn.copy(), sl.copy()))
    launches = ctx.lib.gbfv_kernel_launches() - launches0
    return ms_tot, cells_its, its, launches, ctx.kernel_stats()


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import __graft_entry__ as ge
    if rank == 0 or world == 1:
        ge.build()
    if world > 1:
        dist.barrier()
        ge.build()
    from gbfv import Context, capi
    w = WORKLOADS[args.workload]
    prob = build_problem(args.workload)
    N = prob.num_cells
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    results = {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        ctx = Context(prob, params(prec))
        ctx.save_state()
        ext = torch.cuda.ExternalStream(ctx.stream())
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if name == "mixed" and rank == 0 else None
        if sampler:
            sampler.start()
        ms, cits, its, launches, kst = timed_runs(ctx, w, args.steps, args.warmup, flush, torch, ext)
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        if world > 1:
            t = torch.tensor([ms], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
            c = torch.tensor([cits], dtype=torch.float64, device="cuda")
            dist.all_reduce(c, op=dist.ReduceOp.SUM)
            cits = float(c.item())
        cfg = ctx.solver_config(prec)
        results[name] = dict(ms=ms, cits=cits, its=its, launches=launches, kst=kst, clocks=clocks, ctx=ctx,
                             cfg=cfg)
    # error of the mixed-precision solve against the FP64 solve of the same
    # Newton system (first Newton iteration of the first time step; the FP64
    # GPU path equals the CPU oracle to 1e-8 in the parity tests)
    solve_err = None
    try:
        cm, cf = results["mixed"]["ctx"], results["fp64"]["ctx"]
        dxs = []
        for c in (cm, cf):
            c.restore_state()
            if c.linearize(w["dt"], 0):
                raise RuntimeError("linearization failed")
            _, dx, _ = c.solve(want_dx=True)
            dxs.append(dx)
        solve_err = float(np.max(np.abs(dxs[0] - dxs[1])) / max(np.max(np.abs(dxs[1])), 1e-300))
    except Exception:
        solve_err = None
    # end-to-end through the C ABI with host buffers (mixed form)
    ctx = results["mixed"]["ctx"]
    pv_host = torch.empty(N * 3, dtype=torch.float64, pin_memory=True).numpy()
    m_host = torch.empty(N, dtype=torch.int32, pin_memory=True).numpy()
    out_pv = torch.empty(N * 3, dtype=torch.float64, pin_memory=True).numpy()
    out_m = torch.empty(N, dtype=torch.int32, pin_memory=True).numpy()
    pv_host[:] = prob.init_pv
    m_host[:] = prob.init_meaning
    e2e_s, e2e_cits = 0.0, 0
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.set_solution(pv_host, m_host)
        ctx.lib.gbfv_reset_kernel_stats(ctx.h)
        st, sdt, sn, sl, tl = ctx.time_integration(w["steps"], w["dt"], fixed_dt=True)
        out_pv[:], out_m[:] = ctx.solution()
        e2e_s += time.perf_counter() - t0
        e2e_cits += int(sn.sum()) * N
    # restart file of the final state (the reference's Simulator::serialize
    # layout), written and read back outside the timed regions
    restart_line = None
    if rank == 0:
        import tempfile
        from gbfv import restart
        edges, verts = restart.cartesian_counts((w["nx"], w["ny"], w["nz"]))
        inf = restart.info(edges, verts, time=w["steps"] * w["dt"], time_step_index=w["steps"])
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, restart.restart_file_name(".", "gbfv", inf.time))
            t0 = time.perf_counter()
            ctx.write_restart(path, inf)
            t1 = time.perf_counter()
            ctx.read_restart(path, inf)
            t2 = time.perf_counter()
            restart_line = {"cells": N, "bytes": os.path.getsize(path), "write_ms": (t1 - t0) * 1e3,
                            "read_ms": (t2 - t1) * 1e3, "threads": min(16, os.cpu_count() or 1)}
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
        c = torch.tensor([e2e_cits], dtype=torch.float64, device="cuda")
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        e2e_cits = float(c.item())
    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return 0
    mixed, plain = results["mixed"], results["fp64"]
    value = mixed["cits"] / (mixed["ms"] / 1000.0)
    plain_value = plain["cits"] / (plain["ms"] / 1000.0)
    peak, peak_kind = load_peaks()
    kst = mixed["kst"]
    achieved = kst["solve_bytes"] / (kst["solve_ms"] / 1000.0) / 1e9 if kst["solve_ms"] > 0 else 0.0
    avg_launch_ms = kst["solve_ms"] / max(1, kst["solve_launches"])
    # DRAM traffic of the solver per launch: the ratio of DRAM bytes
    # (dram__bytes_read.sum + dram__bytes_write.sum) to algorithmic bytes of an
    # ncu capture of this workload's solve (profiles/traffic.json), applied to
    # this run's algorithmic bytes per launch
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        try:
            with open(tfile) as f:
                ent = json.load(f).get(args.workload)
            if ent:
                traffic = ent["dram_per_algorithmic_byte"] * kst["solve_bytes"] / max(1, kst["solve_launches"])
        except Exception:
            traffic = None
    lin_ach = kst["linearize_bytes"] / (kst["linearize_ms"] / 1000.0) / 1e9 if kst["linearize_ms"] > 0 else 0.0
    sn0, sl0 = mixed["its"][0]
    spn, spl = plain["its"][0]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mixed["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 residual/Jacobian/update + f32 ILU0/BiCGStab",
        "data": "synthetic (seeded lognormal permeability sigma 1, uniform porosity [0.15,0.30])",
        "config": {"workload": "%s three-phase black-oil, %d cells, 10 time steps x 1 day, "
                               "BiCGStab+ILU0 to 1e-6, Newton tol 1e-6, mixed precision" % (args.workload, N),
                   "cells": N, "time_steps": w["steps"], "precision": "mixed", "l2": "flushed (256 MiB write) "
                   "between timed steps", "parallelism": "replicas" if world > 1 else "single GPU"},
        "plain_fp64": {"value": plain_value, "ms_per_step": plain["ms"] / args.steps,
                       "newton_iterations": spn.tolist(), "linear_iterations": spl.tolist()},
        "mixed_over_plain": value / plain_value,
        "newton_iterations": sn0.tolist(), "linear_iterations": sl0.tolist(),
        "same_newton_iterations": bool(np.array_equal(sn0, spn)),
        "mixed_solve_error_vs_fp64": solve_err,
        "e2e": {"value": e2e_cits / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(N * 3 * 8 + N * 4),
                "d2h_bytes_per_step": int(N * 3 * 8 + N * 4)},
        "gpu_launches": int(mixed["launches"] / args.steps),
        "roofline": {"bound": "hbm", "kernel": "kBicgstab<float,3> (persistent ILU0 + BiCGStab, %s launch of %d blocks)"
                     % (mixed["cfg"]["mode"], mixed["cfg"]["blocks"]),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "avg_launch_ms": avg_launch_ms, "bytes_per_launch": kst["solve_bytes"] / max(1, kst["solve_launches"])},
        "solver_config": {"mixed": mixed["cfg"], "fp64": plain["cfg"]},
        "linearize_roofline": {"achieved": lin_ach, "frac": lin_ach / peak, "ms": kst["linearize_ms"] / args.steps},
        "clocks": mixed["clocks"],
        "restart": restart_line,
    }
    if world == 1 and not args.no_cpu_baseline:
        v, dt, threads = cpu_sample(prob)
        v1, dt1, _ = cpu_sample(prob, iters=1, threads=1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "first 2 Newton iterations of time step 1 (%.1f s)" % dt,
                                "one_thread": {"value": v1, "cores": 1,
                                               "sample": "first Newton iteration of time step 1 (%.1f s)" % dt1}}
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """Initial state of the workload: one linearization (iteration 0) and one
    mixed-precision solve, the unit an ncu capture of the solver covers.
    With --ensemble K: one batched time step of K realizations (clusters of
    2 blocks); prints the batched solve's launches and algorithmic bytes."""
    if args.ensemble > 0:
        probs = ensemble_problems(args.ensemble)  # spawned pool, before any CUDA call
        import __graft_entry__ as ge
        ge.build()
        from gbfv import Batch, capi
        B = Batch(probs, params(capi.PREC_MIXED), cluster_size=2)
        st = B.time_integration(1, ENSEMBLE["dt"])
        s1 = B.stats()
        print(json.dumps({"ensemble": len(probs), "status": st, "solve_launches": s1["solve_launches"],
                          "solve_bytes": s1["solve_bytes"], "solve_ms": s1["solve_ms"],
                          "cells": int(sum(p.num_cells for p in probs))}))
        B.close()
        return 0 if st == 0 else 1
    import __graft_entry__ as ge
    ge.build()
    from gbfv import Context, capi
    w = WORKLOADS[args.workload]
    ctx = Context(build_problem(args.workload), params(capi.PREC_MIXED))
    if ctx.linearize(w["dt"], 0):
        raise RuntimeError("linearization failed")
    lin = ctx.kernel_stats()
    ctx.reset_kernel_stats()
    st, _, it = ctx.solve(want_dx=False)
    ks = ctx.kernel_stats()
    print(json.dumps({"workload": args.workload, "status": st, "iterations": it,
                      "solve_launches": ks["solve_launches"], "solve_bytes": ks["solve_bytes"],
                      "solve_ms": ks["solve_ms"], "linearize_bytes_per_call": lin["linearize_bytes"],
                      "linearize_ms": lin["linearize_ms"]}))
    return 0 if st == 0 else 1


def run_linearizers(args):
    """FvBaseLinearizer::linearize alone on the workload's initial state
    (Newton iteration 1, old storage cached by an iteration-0 call): the AD
    local linearizer and the finite-difference one (forward and central
    differences), device time per call over --steps x 10 calls after
    --warmup, and the CPU oracle on all host threads (one call each)."""
    import __graft_entry__ as ge
    ge.build()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gbfv import Context, capi
    w = WORKLOADS[args.workload]
    prob = build_problem(args.workload)
    out = {"metric": "cells linearized/s", "unit": "cells/s", "workload": args.workload, "cells": prob.num_cells,
           "gpu": {}, "cpu_oracle": {}}
    for name, lin, meth in (("ad", capi.LIN_AD, 1), ("fd_forward", capi.LIN_FD, 1), ("fd_central", capi.LIN_FD, 0)):
        prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, local_linearizer=lin,
                                  numeric_difference_method=meth)
        ctx = Context(prob, prm)
        if ctx.linearize(w["dt"], 0):
            raise RuntimeError("linearization failed")
        for _ in range(max(1, args.warmup)):
            ctx.linearize(w["dt"], 1)
        ctx.reset_kernel_stats()
        n = 10 * max(1, args.steps)
        for _ in range(n):
            if ctx.linearize(w["dt"], 1):
                raise RuntimeError("linearization failed")
        ms = ctx.kernel_stats()["linearize_ms"] / n
        out["gpu"][name] = {"ms": ms, "value": prob.num_cells / (ms / 1e3)}
        ctx.close()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    for name, lin in (("ad", capi.LIN_AD), ("fd_forward", capi.LIN_FD)):
        orc = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, local_linearizer=lin))
        orc.linearize(w["dt"], 0)
        t0 = time.perf_counter()
        orc.linearize(w["dt"], 1)
        dt = time.perf_counter() - t0
        out["cpu_oracle"][name] = {"ms": dt * 1e3, "value": prob.num_cells / dt, "cores": threads}
    print(json.dumps(out))
    return 0


ENSEMBLE = dict(lo=10000, hi=200000, sigma=(0.5, 1.5), seed=1000, steps=2, dt=250.0)


def _member(args):
    n, seed, sigma = args
    from gbfv import problems
    return problems.ensemble_member(n, seed, sigma)


def ensemble_problems(count, rank=0, world=1):
    """Seeded ensemble: cell counts uniform in [10k, 200k], lognormal
    permeability with sigma uniform in [0.5, 1.5] (built in a spawned pool).
    With several ranks each builds the members assigned to it by size."""
    import multiprocessing as mp
    from gbfv import replicas
    rng = np.random.default_rng(ENSEMBLE["seed"])
    sizes = rng.integers(ENSEMBLE["lo"], ENSEMBLE["hi"] + 1, count)
    sig = rng.uniform(*ENSEMBLE["sigma"], count)
    mine = replicas.assign([int(n) for n in sizes], world)[rank]
    jobs = [(int(sizes[i]), ENSEMBLE["seed"] + i, float(sig[i])) for i in mine]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        return pool.map(_member, jobs, chunksize=1)


def run_ensemble(args):
    """Batched ensemble: all realizations advanced together by gbfv_batch
    (one launch per phase, one persistent solve launch per round, captured
    CUDA graphs).  value = sum over systems of Newton iterations x cells /
    device time of the whole batch; one_at_a_time = the same systems solved
    one after another through single contexts (a sample of them), in the
    mixed form and (one_at_a_time_plain_fp64) in plain FP64, whose ratio to
    the batched value is batched_mixed_over_plain_fp64."""
    rank, world, local = dist_env()
    t0 = time.time()
    probs = ensemble_problems(args.ensemble, rank, world)  # before any CUDA call (spawned pool)
    t_build = time.time() - t0
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as ge
    if rank == 0:
        ge.build()
    if world > 1:
        dist.barrier()
    ge.build()
    from gbfv import Batch, Context, capi, replicas
    prm = params(capi.PREC_MIXED)
    t0 = time.time()
    B = Batch(probs, prm)
    t_create = time.time() - t0
    cluster, tune_ms = B.autotune(ENSEMBLE["dt"])
    for c in B.systems:
        c.save_state()
    ext = torch.cuda.ExternalStream(B.stream())
    Ns = np.array([p.num_cells for p in probs])

    def one_run():
        for c in B.systems:
            c.restore_state()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        st = B.time_integration(ENSEMBLE["steps"], ENSEMBLE["dt"])
        e1.record(ext)
        e1.synchronize()
        if st:
            raise RuntimeError("batched run failed %d" % st)
        cits = sum(int(B.report(i)[2].sum()) * int(Ns[i]) for i in range(len(probs)))
        return e0.elapsed_time(e1), cits

    for _ in range(args.warmup):
        one_run()
    s0 = B.stats()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    ms_tot, cits_tot = 0.0, 0
    for _ in range(args.steps):
        ms, cits = one_run()
        ms_tot += ms
        cits_tot += cits
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    s1 = B.stats()
    # whole job: the slowest rank's time, all ranks' work (no data-path collective)
    ms_tot, cits_tot = replicas.reduce_timing(ms_tot, cits_tot, device="cuda")
    value = cits_tot / (ms_tot / 1000.0)
    if rank != 0:
        B.close()
        dist.barrier()
        dist.destroy_process_group()
        return 0
    newton = [B.report(i)[2].tolist() for i in range(len(probs))]
    # one at a time: a sample of the same systems through single contexts,
    # in the mixed form and in the plain FP64 form
    sample = list(range(0, len(probs), max(1, len(probs) // 8)))[:8]
    B.close()

    def one_at_a_time(prm1):
        ms, cits = 0.0, 0
        for i in sample:
            ctx = Context(probs[i], prm1)
            ctx.time_integration(ENSEMBLE["steps"], ENSEMBLE["dt"])  # warm-up incl. autotuning
            ctx.set_solution(probs[i].init_pv, probs[i].init_meaning)
            ext1 = torch.cuda.ExternalStream(ctx.stream())
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext1)
            st, sdt, sn, sl, tl = ctx.time_integration(ENSEMBLE["steps"], ENSEMBLE["dt"])
            e1.record(ext1)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            cits += int(sn.sum()) * probs[i].num_cells
            ctx.close()
        return cits / (ms / 1000.0)

    one_value = one_at_a_time(prm)
    one_fp64 = one_at_a_time(params(capi.PREC_FP64))
    peak, peak_kind = load_peaks()
    solve_ms = s1["solve_ms"] - s0["solve_ms"]
    solve_bytes = s1["solve_bytes"] - s0["solve_bytes"]
    achieved = solve_bytes / (solve_ms / 1000.0) / 1e9 if solve_ms > 0 else 0.0
    solve_launches = max(1, s1["solve_launches"] - s0["solve_launches"])
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            ent = json.load(f).get("ensemble")
        if ent:  # DRAM bytes per algorithmic byte of an ncu capture of the batched solve
            traffic = ent["dram_per_algorithmic_byte"] * solve_bytes / solve_launches
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_tot / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 residual/Jacobian/update + f32 ILU0/BiCGStab",
        "data": "synthetic (seeded ensemble: cells uniform 10k-200k, lognormal permeability sigma 0.5-1.5)",
        "config": {"workload": "ensemble-%d two-phase immiscible realizations, %d cells in total, %d time steps "
                               "x %.0f s each, BiCGStab+ILU0 to 1e-6, mixed precision, batched"
                               % (len(probs), int(Ns.sum()), ENSEMBLE["steps"], ENSEMBLE["dt"]),
                   "systems": len(probs), "cells_total": int(Ns.sum()), "cells_min": int(Ns.min()),
                   "cells_max": int(Ns.max()), "l2": "inputs larger than L2 (%.1f GB of state)" % (Ns.sum() * 1.5e-6),
                   "parallelism": "single GPU"},
        "batch": {"cluster_size": cluster, "num_clusters": s1["num_clusters"], "tune_ms": tune_ms.tolist(),
                  "rounds_per_step": (s1["rounds"] - s0["rounds"]) / args.steps,
                  "graph_launches_per_step": (s1["graph_launches"] - s0["graph_launches"]) / args.steps,
                  "build_s": t_build, "create_s": t_create},
        "one_at_a_time": {"value": one_value, "systems_sampled": len(sample)},
        "one_at_a_time_plain_fp64": {"value": one_fp64, "systems_sampled": len(sample)},
        "batched_over_one_at_a_time": (value / world) / one_value,
        "batched_mixed_over_plain_fp64": (value / world) / one_fp64,
        "gpu_launches": int((s1["kernel_launches"] - s0["kernel_launches"]) / args.steps),
        "newton_iterations_first_systems": newton[:4],
        "roofline": {"bound": "hbm", "kernel": "kBicgstabBatch<float,2> (batched persistent ILU0 + BiCGStab)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_kind": peak_kind},
        "clocks": clocks,
    }
    if world > 1:
        line["n_gpus"] = world
        line["config"]["parallelism"] = "replicas (systems assigned to ranks by size)"
        line["config"]["systems_on_rank0"] = len(probs)
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


SERVE = dict(lo=20000, hi=1000000, pool=12, requests=24, rates=(50, 200, 1000, 2000), seed=2024, dt=86400.0,
             capacity=16, cluster=8, lanes=((150000, 12, 4),))


def _serve_problem(job):
    n, seed = job
    from gbfv import problems
    nz = max(4, int(round(n ** (1.0 / 3.0) / 1.5)))
    nxy = max(4, int(round(math.sqrt(n / nz))))
    return problems.blackoil(nxy, nxy, nz, seed=seed)


def run_serve(args):
    """Served stream: requests (one black-oil time step each, grids
    log-uniform in 20k-1M cells, drawn from a seeded pool) arrive as a
    Poisson process; the server admits them by HBM footprint into slots and
    batches them on arrival (continuous batching, mixed precision).  Reported
    per arrival rate: p50/p99 latency (arrival -> state on the host) and
    throughput, beside the plain-FP64 one-at-a-time GPU path on the same
    traces."""
    import multiprocessing as mp
    rng = np.random.default_rng(SERVE["seed"])
    sizes = np.exp(rng.uniform(math.log(SERVE["lo"]), math.log(SERVE["hi"]), SERVE["pool"])).astype(int)
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        probs = pool.map(_serve_problem, [(int(n), SERVE["seed"] + i) for i, n in enumerate(sizes)], chunksize=1)
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as ge
    ge.build()
    from gbfv import capi
    from gbfv.serving import (LanedServer, Request, Server, latency_summary, serve, serve_laned,
                              serve_one_at_a_time)
    prm = params(capi.PREC_MIXED)
    big = max(p.num_cells for p in probs)

    def trace(rate, seed):
        r = np.random.default_rng(seed)
        t = np.cumsum(r.exponential(1.0 / rate, SERVE["requests"]))
        return [Request(probs[i % len(probs)], steps=1, dt=SERVE["dt"], arrival=float(a), rid=i)
                for i, a in enumerate(t)]

    # one lane: every request in one batch
    srv = Server(capi.MODEL_BLACKOIL_3P, prm, capacity=SERVE["capacity"], cluster_size=SERVE["cluster"],
                 max_cells=big)
    serve(srv, trace(1000, 1)[:4])  # warm-up: module load, graphs, pinned buffers
    top_rate = SERVE["rates"][-1]
    single = latency_summary(serve(srv, trace(top_rate, top_rate)))
    srv.close()
    # size lanes: requests up to 150k cells in clusters of 4, larger ones in
    # clusters of 16, side by side on their own streams
    laned = LanedServer(capi.MODEL_BLACKOIL_3P, prm, lanes=SERVE["lanes"] + ((big, 4, 16),))
    serve_laned(laned, trace(1000, 1)[:6])
    sampler = ClockSampler(0)
    sampler.start()
    served = {}
    for rate in SERVE["rates"]:
        reqs = serve_laned(laned, trace(rate, rate))
        served[str(rate)] = latency_summary(reqs)
    clocks = sampler.stop()
    laned.close()
    base = {}
    for rate in (SERVE["rates"][0], SERVE["rates"][-1]):
        reqs = serve_one_at_a_time(trace(rate, rate), params(capi.PREC_FP64))
        base[str(rate)] = latency_summary(reqs)
    top = str(SERVE["rates"][-1])
    line = {
        "metric": METRIC, "value": served[top]["cell_newton_its_per_s"], "unit": UNIT, "n_gpus": 1,
        "steps": len(SERVE["rates"]), "warmup": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 residual/Jacobian/update + f32 ILU0/BiCGStab",
        "data": "synthetic (seeded black-oil grids, cells log-uniform 20k-1M, lognormal permeability sigma 1)",
        "config": {"workload": "served stream of single-time-step black-oil solves, Poisson arrivals at %s req/s, "
                               "%d requests per rate, continuous batching, admission by HBM footprint, "
                               "mixed precision" % (list(SERVE["rates"]), SERVE["requests"]),
                   "pool_cells": [int(p.num_cells) for p in probs],
                   "lanes": "cells <= 150k: 12 slots, clusters of 4; larger: 4 slots, clusters of 16",
                   "parallelism": "single GPU"},
        "served": served,
        "one_lane_at_top_rate": single,
        "one_at_a_time_fp64": base,
        "p50_ms": served[top]["p50_ms"], "p99_ms": served[top]["p99_ms"],
        "clocks": clocks,
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.profile_case:
        return run_profile_case(args)
    if args.linearizers:
        return run_linearizers(args)
    if args.serve:
        return run_serve(args)
    if args.ensemble > 0:
        return run_ensemble(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
