#!/usr/bin/env python
"""Benchmark: cell-Newton-iterations/s of the ECFV/TPFA linearization +
BiCGStab/ILU0 Newton solve.

Default workload: three-phase black-oil on 100x100x100 (1M cells, 3x3
blocks), 10 time steps of 1 day, BiCGStab + ILU(0) to 1e-6 relative residual,
Newton tolerance 1e-6.  One bench step = one time step of that run; the steps
cycle through the run's 10 time steps, the initial state being restored on
the device before the first of them.  value = sum over the timed steps of
Newton iterations x cells / device time, for the mixed-precision form (FP64
residual/Jacobian/update/outer residual, FP32 ILU0 + FP32 BiCGStab inside FP64
iterative refinement).  Beside it: the plain FP64 form on the same steps, the
same two forms on 100x100x20 (200k cells), the 48x32 lens (30 steps, FP64)
with the CPU oracle, the mixed solve's error against the FP64 solve of the
same system for every solve of time step 1, and a matched sample: the GPU's
rate over exactly the Newton iterations the reference arm times.

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
DEFAULT_WORKLOAD = "blackoil-100x100x100"
SECONDARY_WORKLOAD = "blackoil-100x100x20"
METRIC = "cell-Newton-iters/s (mixed vs plain FP64, same tol); served solve p50/p99 ms"
UNIT = "cell-Newton-iters/s"
LENS = dict(nx=48, ny=32, steps=30, dt=250.0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="only the headline workload (no 100x100x20 and lens lines)")
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


def workload_config(wl, precision="mixed"):
    """The `config` both arms print (the reference arm times a bounded
    sample of this same workload and says which in cpu_baseline.sample)."""
    w = WORKLOADS[wl]
    N = w["nx"] * w["ny"] * w["nz"]
    return {"workload": "%s three-phase black-oil, %d cells, %d time steps x 1 day, BiCGStab+ILU0 to 1e-6, "
                        "Newton tol 1e-6, %s precision; one bench step = one time step (cycled)"
                        % (wl, N, w["steps"], precision),
            "cells": N, "time_steps": w["steps"], "precision": precision,
            "l2": "flushed (256 MiB write) between timed steps", "parallelism": "single GPU"}


class NewtonStepper:
    """The workload's Newton iterations one at a time, in the order
    NewtonMethod::apply (newtonmethod.hh:228-438) runs them inside the
    fixed-dt time loop: iteration j of a time step linearizes at the current
    state (j = 0 also caches the old storage, the time-level advance of the
    storage term), takes the Newton error and, unless the step has converged
    (j >= 1 and error <= tolerance), solves and updates.  Drives a
    gbfv.Context or an oracle.Oracle (the same method names)."""

    def __init__(self, system, dt, tol, max_iter=20):
        self.s, self.dt, self.tol, self.max_iter = system, dt, tol, max_iter
        self.step, self.j, self.newton = 0, 0, []

    def _error(self):
        e = self.s.newton_error()
        if isinstance(e, tuple):
            st, e = e
            if st:
                raise RuntimeError("newton_error failed %d" % st)
        return e

    def next(self, want_dx=False):
        """One Newton iteration; returns (time step, iteration, solved, dx, linear iterations)."""
        st = self.s.linearize(self.dt, self.j)
        if st:
            raise RuntimeError("linearize failed %d" % st)
        err = self._error()
        here = (self.step, self.j)
        if self.j >= 1 and err <= self.tol:
            self.newton.append(self.j + 1)
            self.step, self.j = self.step + 1, 0
            return here + (False, None, 0)
        if self.j + 1 >= self.max_iter:
            raise RuntimeError("Newton did not converge in %d iterations" % self.max_iter)
        if want_dx or not hasattr(self.s, "stream"):
            st, dx, it = self.s.solve()
        else:
            st, dx, it = self.s.solve(want_dx=False)
        if st:
            raise RuntimeError("solve failed %d" % st)
        st, _ = self.s.newton_update()
        if st:
            raise RuntimeError("newton_update failed %d" % st)
        self.j += 1
        return here + (True, dx, it)


def cpu_sample(prob, iters=1, threads=None):
    """The oracle (the reference algorithm restated on the CPU) on the first
    `iters` Newton iterations of the first time step: OpenMP over elements in
    the linearization, sequential BiCGStab/ILU0 (as the reference)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    orc = O.Oracle(prob, params(0))
    ns = NewtonStepper(orc, 86400.0, params(0).newton_tolerance)
    t0 = time.perf_counter()
    for _ in range(iters):
        ns.next()
    dt = time.perf_counter() - t0
    orc.close()
    return iters * prob.num_cells / dt, dt, threads


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm restated on
    the CPU; the reference itself cannot be built here) on all host threads,
    on the same workload and config as our arm.  Each bench step is one Newton
    iteration of the workload's run, in the run's order (time step 1's
    iterations, then time step 2's, ...): W untimed, then K timed.  Our arm's
    matched_sample times exactly these iterations on the GPU."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    w = WORKLOADS[args.workload]
    prob = build_problem(args.workload)
    orc = O.Oracle(prob, params(0))
    ns = NewtonStepper(orc, w["dt"], params(0).newton_tolerance)
    for _ in range(args.warmup):
        ns.next()
    tot, done = 0.0, []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        done.append(ns.next()[:2])
        tot += time.perf_counter() - t0
    orc.close()
    value = args.steps * prob.num_cells / tot
    sample = ("Newton iterations %d..%d of the workload's run (time step, iteration): %s; one per step, the "
              "first %d untimed" % (args.warmup + 1, args.warmup + args.steps, done, args.warmup))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lognormal permeability sigma 1, uniform porosity [0.15,0.30])",
        "config": workload_config(args.workload),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def timed_time_steps(ctx, w, steps, warmup, flush, torch, ext):
    """Device time of `steps` time steps of the workload, after `warmup`
    untimed ones; the steps cycle through the run's time steps, the initial
    state restored (on the device, outside the timed region) before each
    cycle's first step, and L2 flushed before every timed step."""
    n = w["steps"]
    for k in range(warmup):
        if k % n == 0:
            ctx.restore_state()
        st, _, _, _, _ = ctx.time_integration(1, w["dt"], fixed_dt=True)
        if st:
            raise RuntimeError("warm-up step failed %d" % st)
    ms_tot, cells_its, newton, linear = 0.0, 0, [], []
    launches0 = ctx.lib.gbfv_kernel_launches()
    ctx.reset_kernel_stats()
    for k in range(steps):
        if k % n == 0:
            ctx.restore_state()
        with torch.cuda.stream(ext):
            flush.zero_()  # write a buffer larger than L2 between timed steps
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        st, sdt, sn, sl, tl = ctx.time_integration(1, w["dt"], fixed_dt=True)
        e1.record(ext)
        e1.synchronize()
        if st:
            raise RuntimeError("timed step failed %d" % st)
        ms_tot += e0.elapsed_time(e1)
        cells_its += int(sn[0]) * ctx.N
        newton.append(int(sn[0]))
        linear.append(int(sl[0]))
    launches = ctx.lib.gbfv_kernel_launches() - launches0
    return dict(ms=ms_tot, cits=cells_its, newton=newton, linear=linear, launches=launches,
                kst=ctx.kernel_stats())


def newton_iteration_ms(ctx, w, count, torch, ext):
    """Device time of each of the first `count` Newton iterations of the
    workload's run (from the initial state), driven one at a time through the
    C ABI as NewtonMethod::apply runs them; returns [(time step, iteration,
    ms)]."""
    ctx.restore_state()
    ns = NewtonStepper(ctx, w["dt"], params(0).newton_tolerance)
    out = []
    for _ in range(count):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s, j, _, _, _ = ns.next()
        e1.record(ext)
        e1.synchronize()
        out.append((s, j, e0.elapsed_time(e1)))
    return out


def mixed_solve_errors(ctx, w, torch):
    """Every solve of time step 1 (mixed-precision run from the initial
    state): the same Newton system solved in plain FP64 and in the mixed
    form; error = max |dx_mixed - dx_fp64| / max |dx_fp64|.  The mixed dx is
    the one applied (it is the context's last solve)."""
    from gbfv import capi
    ctx.restore_state()
    pm, pf = params(capi.PREC_MIXED), params(capi.PREC_FP64)
    ns = NewtonStepper(ctx, w["dt"], pm.newton_tolerance)
    errs = []
    while ns.step == 0:
        st = ctx.linearize(w["dt"], ns.j)
        st2, err = ctx.newton_error()
        if st or st2:
            raise RuntimeError("linearize failed")
        if ns.j >= 1 and err <= ns.tol:
            break
        ctx.set_params(pf)
        st, dxf, _ = ctx.solve(want_dx=True)
        ctx.set_params(pm)
        st2, dxm, _ = ctx.solve(want_dx=True)
        if st or st2:
            raise RuntimeError("solve failed")
        errs.append(float(np.max(np.abs(dxm - dxf)) / max(np.max(np.abs(dxf)), 1e-300)))
        ctx.newton_update()
        ns.j += 1
    return errs


def lens_line(torch, vcfv=False, blackoil=False):
    """The 48x32 lens (lensproblem.hh:227-627), 30 time steps from dt0 = 250 s
    with the reference's dt control, FP64, BiCGStab + ILU(0) to 1e-6: the GPU
    (device time of the whole run, after one untimed run) beside the oracle
    (all host threads, and one).  vcfv: the same problem on the vertex-
    centred discretization with P1 gradients (lens_immiscible_vcfv_ad.cc),
    49x33 vertices, the 9-point Jacobian through the general block ILU(0).
    blackoil: the black-oil vertical section on the vertex-centred grid
    (reservoir_blackoil_vcfv's 2D configuration, 41x21 vertices, wells as
    constraint vertices), 10 daily steps."""
    from gbfv import Context, capi, problems
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    steps, dt0, fixed = LENS["steps"], LENS["dt"], False
    if blackoil:
        prob = problems.blackoil_vcfv(40, 20)
        prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
        steps, dt0, fixed = 10, 86400.0, True
    else:
        prob = problems.lens_vcfv(LENS["nx"], LENS["ny"]) if vcfv else problems.lens(LENS["nx"], LENS["ny"])
        prm = capi.default_params(linear_tolerance=1e-6)
    ctx = Context(prob, prm)
    ctx.save_state()
    ext = torch.cuda.ExternalStream(ctx.stream())
    ctx.time_integration(steps, dt0, fixed_dt=fixed)
    ctx.restore_state()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    st, sdt, sn, sl, _ = ctx.time_integration(steps, dt0, fixed_dt=fixed)
    e1.record(ext)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    ctx.close()
    cits = int(sn.sum()) * prob.num_cells
    if blackoil:
        what = ("blackoil-vcfv-40x20 three-phase black-oil vertical section, vertex-centred, P1 gradients, "
                "861 vertices, wells as constraint vertices, 10 steps of 1 day")
    else:
        what = ("lens-vcfv-48x32 two-phase immiscible (VG), vertex-centred, P1 gradients, 1617 vertices"
                if vcfv else "lens-48x32 two-phase immiscible (VG), 1536 cells") + ", 30 time steps from 250 s"
    out = {"workload": what + ", FP64, BiCGStab+ILU0 to 1e-6",
           "unit": "dof-Newton-iters/s", "status": st, "value": cits / (ms / 1e3), "ms": ms,
           "newton_iterations": int(sn.sum()), "linear_iterations": int(sl.sum()), "final_dt": float(sdt[-1])}
    O.build()
    for name, threads in (("cpu_oracle", os.cpu_count() or 1), ("cpu_oracle_one_thread", 1)):
        O.set_threads(threads)
        orc = O.Oracle(prob, prm)
        t0 = time.perf_counter()
        sto, _, sno, _, _ = orc.time_integration(steps, dt0, fixed_dt=fixed)
        dt = time.perf_counter() - t0
        orc.close()
        out[name] = {"value": int(sno.sum()) * prob.num_cells / dt, "s": dt, "cores": threads,
                     "same_newton_iterations": bool(np.array_equal(sno, sn))}
    return out


def solver_kernel_name(cfg):
    """The persistent solve kernel a solver configuration runs."""
    if cfg["mode"].startswith("gilu"):
        return ("kGiluBicgstab<float,3,%s> (persistent block ILU(0) + BiCGStab, %s sweeps, cooperative grid of "
                "%d blocks)" % ("tagged" if "tagged" in cfg["mode"] else "level",
                               "tagged" if "tagged" in cfg["mode"] else "level-barrier", cfg["blocks"]))
    return "kBicgstab<float,3> (persistent ILU0 + BiCGStab, %s launch of %d blocks)" % (cfg["mode"], cfg["blocks"])


def solver_traffic(wl, kst, kernel=None):
    """DRAM traffic of the solver per launch: the ratio of DRAM bytes
    (dram__bytes_read.sum + dram__bytes_write.sum) to algorithmic bytes of an
    ncu capture of this workload's solve (profiles/traffic.json), applied to
    this run's algorithmic bytes per launch."""
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(tfile) as f:
            ent = json.load(f).get(wl)
        # the capture of the kernel this run's solves used
        if ent and kernel and ent.get("kernel", "").split("<")[0] != kernel.split("<")[0]:
            ent = None
        if ent:
            kind = ent.get("traffic_kind", "scaled from a capture of the cluster launch of the same kernel body")
            return ent["dram_per_algorithmic_byte"] * kst["solve_bytes"] / max(1, kst["solve_launches"]), kind
    except Exception:
        pass
    return None, None


def run_workload(wl, args, flush, torch, world, sampler_local=None):
    """Both forms of one workload: timed time steps, solver configuration."""
    from gbfv import Context, capi
    w = WORKLOADS[wl]
    prob = build_problem(wl)
    out = {"prob": prob}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        ctx = Context(prob, params(prec))
        ctx.save_state()
        ext = torch.cuda.ExternalStream(ctx.stream())
        torch.cuda.synchronize()
        sampler = ClockSampler(sampler_local) if (name == "mixed" and sampler_local is not None) else None
        if sampler:
            sampler.start()
        r = timed_time_steps(ctx, w, args.steps, args.warmup, flush, torch, ext)
        torch.cuda.synchronize()
        r["clocks"] = sampler.stop() if sampler else None
        r["cfg"] = ctx.solver_config(prec)
        r["ctx"], r["ext"] = ctx, ext
        out[name] = r
    return out


# one-way hop of a level's result to a consumer CTA of the cluster
# (st.async of 16 B counted on the receiver's mbarrier), measured by a
# micro-benchmark on a GB300: the least a dependent level step can take
LEVEL_HOP_CYCLES = 370


def latency_floor(w, kst, clocks):
    """Latency roofline of the ILU(0) solver: exact ILU(0) fixes the
    wavefront level count (nx + ny + nz - 2 on these grids), every BiCGStab
    iteration runs two preconditioner applications of a forward and a
    backward sweep over all levels, and no level step can be shorter than
    one hop of its result to the next level's CTA.  The hop is the
    cluster's distributed-shared-memory hop; the tagged sweeps pass a
    result through L2, which takes longer, so the floor bounds both.
    floor_ms = iterations x 4 x levels x hop; frac = floor_ms / the
    solver's measured time."""
    levels = w["nx"] + w["ny"] + w["nz"] - 2
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    hop_us = LEVEL_HOP_CYCLES / mhz
    floor_ms = kst["solve_iterations"] * 4 * levels * hop_us / 1e3
    return {"levels_per_sweep": levels, "sweeps_per_iteration": 4, "hop_cycles": LEVEL_HOP_CYCLES,
            "hop_us": hop_us, "iterations": int(kst["solve_iterations"]), "floor_ms": floor_ms,
            "solver_ms": kst["solve_ms"], "frac": floor_ms / kst["solve_ms"] if kst["solve_ms"] > 0 else None}


def amg_line(wl, args, flush, torch, ilu_value=None):
    """The workload through the AMG backend (linear_solver = LINSOLVER_AMG,
    the reference's ParallelAmgBackend) in mixed precision: the same timed
    time steps as the headline, the hierarchy built during the warm-up."""
    from gbfv import Context, capi
    w = WORKLOADS[wl]
    prob = build_problem(wl)
    prm = params(capi.PREC_MIXED)
    prm.linear_solver = capi.LINSOLVER_AMG
    ctx = Context(prob, prm)
    ctx.save_state()
    ext = torch.cuda.ExternalStream(ctx.stream())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, _, _, _, _ = ctx.time_integration(1, w["dt"], fixed_dt=True)  # builds the hierarchy
    setup_s = time.perf_counter() - t0
    if st:
        raise RuntimeError("AMG first step failed %d" % st)
    r = timed_time_steps(ctx, w, args.steps, max(0, args.warmup - 1), flush, torch, ext)
    value = r["cits"] / (r["ms"] / 1e3)
    kst = r["kst"]
    peak, peak_kind = load_peaks()
    achieved = kst["solve_bytes"] / (kst["solve_ms"] / 1e3) / 1e9 if kst["solve_ms"] > 0 else 0.0
    sizes, colors = ctx.amg_levels()
    ctx.close()
    out = {"value": value, "unit": UNIT, "ms_per_step": r["ms"] / args.steps,
           "newton_iterations": r["newton"], "linear_iterations": r["linear"],
           "first_step_with_setup_s": setup_s,
           "levels": [int(v) for v in sizes], "colors": [int(v) for v in colors],
           "roofline": {"kernel": "kAmgBicgstab<float,3> (persistent BiCGStab + AMG V-cycle, cooperative grid)",
                        "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "peak_kind": peak_kind, "solve_ms_per_step": kst["solve_ms"] / args.steps},
           "what": "mixed precision through the AMG backend (BiCGStab + aggregation AMG V-cycle, "
                   "ParallelAmgBackend), same tolerances and time steps as the ILU(0) headline"}
    if ilu_value:
        out["amg_over_ilu0"] = value / ilu_value
    return out


def ensemble_leg(count, torch):
    """A compact C4 line inside the default benchmark: `count` seeded
    two-phase realizations (10k-200k cells) advanced together by the batched
    path in mixed precision, the same batch in plain FP64, and a sample of 4
    of them one at a time in plain FP64 -- the form the batched mixed rate is
    compared with (batched_mixed_over_plain_fp64).  One untimed run of each,
    then one timed run of ENSEMBLE["steps"] time steps."""
    from gbfv import Batch, Context, capi
    probs = ensemble_problems(count)
    Ns = np.array([p.num_cells for p in probs])

    def batched(prec):
        B = Batch(probs, params(prec))
        B.autotune(ENSEMBLE["dt"])
        for c in B.systems:
            c.save_state()
        ext = torch.cuda.ExternalStream(B.stream())
        out = None
        for _ in range(2):
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
            out = (cits / (e0.elapsed_time(e1) / 1000.0), [B.report(i)[2].tolist() for i in range(len(probs))])
        B.close()
        return out

    mixed, newton = batched(capi.PREC_MIXED)
    fp64, newton64 = batched(capi.PREC_FP64)
    ms, cits = 0.0, 0
    for i in range(0, len(probs), max(1, len(probs) // 4))[:4]:
        ctx = Context(probs[i], params(capi.PREC_FP64))
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
    one_fp64 = cits / (ms / 1000.0)
    return {"systems": count, "cells_total": int(Ns.sum()), "value": mixed, "unit": UNIT,
            "batched_plain_fp64": fp64, "one_at_a_time_plain_fp64": one_fp64,
            "batched_mixed_over_plain_fp64": mixed / one_fp64, "batched_mixed_over_batched_plain_fp64": mixed / fp64,
            "same_newton_iterations": newton == newton64,
            "what": "two-phase realizations with 10k-200k cells, %d time steps x %g s, batched (device-driven "
                    "Newton rounds, one graph launch each); the full 256-member line is bench.py --ensemble 256"
                    % (ENSEMBLE["steps"], ENSEMBLE["dt"])}


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
    from gbfv import replicas
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    if world > 1:
        dist.barrier()
    head = run_workload(args.workload, args, flush, torch, world, sampler_local=local if rank == 0 else None)
    w = WORKLOADS[args.workload]
    prob = head["prob"]
    N = prob.num_cells
    mixed, plain = head["mixed"], head["fp64"]
    ms_m, cits_m = replicas.reduce_timing(mixed["ms"], mixed["cits"], device="cuda") if world > 1 \
        else (mixed["ms"], mixed["cits"])
    ms_f, cits_f = replicas.reduce_timing(plain["ms"], plain["cits"], device="cuda") if world > 1 \
        else (plain["ms"], plain["cits"])
    # end-to-end through the C ABI with host buffers (mixed form): every step
    # copies the state in from pinned host memory and the result back out
    ctx = mixed["ctx"]
    pv_host = torch.empty(N * 3, dtype=torch.float64, pin_memory=True).numpy()
    m_host = torch.empty(N, dtype=torch.int32, pin_memory=True).numpy()
    pv_host[:] = prob.init_pv
    m_host[:] = prob.init_meaning
    e2e_s, e2e_cits = 0.0, 0
    for k in range(args.steps):
        if k % w["steps"] == 0:
            pv_host[:] = prob.init_pv
            m_host[:] = prob.init_meaning
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.set_solution(pv_host, m_host)
        st, sdt, sn, sl, tl = ctx.time_integration(1, w["dt"], fixed_dt=True)
        pv_host[:], m_host[:] = ctx.solution()
        e2e_s += time.perf_counter() - t0
        if st:
            raise RuntimeError("e2e step failed %d" % st)
        e2e_cits += int(sn[0]) * N
    if world > 1:
        e2e_ms, e2e_cits = replicas.reduce_timing(e2e_s * 1e3, e2e_cits, device="cuda")
        e2e_s = e2e_ms / 1e3
    if rank != 0:
        dist.barrier()
        dist.destroy_process_group()
        return 0
    # per-solve error of the mixed form against FP64 on the same systems
    solve_errs = mixed_solve_errors(ctx, w, torch)
    # matched sample: the Newton iterations the reference arm times
    matched = {}
    count = args.warmup + args.steps
    for name in ("mixed", "fp64"):
        it_ms = newton_iteration_ms(head[name]["ctx"], w, count, torch, head[name]["ext"])
        timed = it_ms[args.warmup:]
        matched[name] = {"value": len(timed) * N / (sum(t[2] for t in timed) / 1e3),
                         "iterations": [[t[0], t[1]] for t in timed]}
    # restart file of the final state (the reference's Simulator::serialize
    # layout), written and read back outside the timed regions
    restart_line = None
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
    value = cits_m / (ms_m / 1000.0)
    plain_value = cits_f / (ms_f / 1000.0)
    peak, peak_kind = load_peaks()
    kst = mixed["kst"]
    achieved = kst["solve_bytes"] / (kst["solve_ms"] / 1000.0) / 1e9 if kst["solve_ms"] > 0 else 0.0
    avg_launch_ms = kst["solve_ms"] / max(1, kst["solve_launches"])
    traffic, traffic_kind = solver_traffic(args.workload, kst, solver_kernel_name(mixed["cfg"]))
    lin_ach = kst["linearize_bytes"] / (kst["linearize_ms"] / 1000.0) / 1e9 if kst["linearize_ms"] > 0 else 0.0
    for name in ("mixed", "fp64"):
        head[name]["ctx"].close()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mixed["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 residual/Jacobian/update + f32 ILU0/BiCGStab",
        "data": "synthetic (seeded lognormal permeability sigma 1, uniform porosity [0.15,0.30])",
        "config": workload_config(args.workload),
        "plain_fp64": {"value": plain_value, "ms_per_step": plain["ms"] / args.steps,
                       "newton_iterations": plain["newton"], "linear_iterations": plain["linear"],
                       "dtype": "f64"},
        "mixed_over_plain": value / plain_value,
        "newton_iterations": mixed["newton"], "linear_iterations": mixed["linear"],
        "same_newton_iterations": mixed["newton"] == plain["newton"],
        "mixed_solve_error_vs_fp64": {"time_step": 1, "per_solve": solve_errs,
                                      "what": "max|dx_mixed - dx_fp64| / max|dx_fp64| of the same Newton "
                                              "system; the FP64 path equals the oracle's solve to rounding"},
        "matched_sample": {"value": matched["mixed"]["value"], "plain_fp64": matched["fp64"]["value"],
                           "unit": UNIT, "iterations": matched["mixed"]["iterations"],
                           "what": "GPU rate over exactly the Newton iterations (time step, iteration) the "
                                   "reference arm times, driven one at a time through the C ABI"},
        "e2e": {"value": e2e_cits / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(N * 3 * 8 + N * 4),
                "d2h_bytes_per_step": int(N * 3 * 8 + N * 4)},
        "gpu_launches": int(mixed["launches"] / args.steps),
        "roofline": {"bound": "hbm", "kernel": solver_kernel_name(mixed["cfg"]),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_kind": traffic_kind, "peak_kind": peak_kind,
                     "avg_launch_ms": avg_launch_ms,
                     "bytes_per_launch": kst["solve_bytes"] / max(1, kst["solve_launches"]),
                     "latency_floor": latency_floor(w, kst, mixed["clocks"])},
        "solver_config": {"mixed": mixed["cfg"], "fp64": plain["cfg"]},
        "linearize_roofline": {"achieved": lin_ach, "frac": lin_ach / peak, "ms": kst["linearize_ms"] / args.steps},
        "clocks": mixed["clocks"],
        "restart": restart_line,
    }
    # the AMG backend on the same workload
    if not args.headline_only:
        line["amg"] = amg_line(args.workload, args, flush, torch, value)
    # the same two forms on the 200k-cell grid
    if args.workload != SECONDARY_WORKLOAD and not args.headline_only:
        sec = run_workload(SECONDARY_WORKLOAD, args, flush, torch, 1)
        sm, sf = sec["mixed"], sec["fp64"]
        v2m, v2f = sm["cits"] / (sm["ms"] / 1e3), sf["cits"] / (sf["ms"] / 1e3)
        k2 = sm["kst"]
        a2 = k2["solve_bytes"] / (k2["solve_ms"] / 1e3) / 1e9 if k2["solve_ms"] > 0 else 0.0
        line[SECONDARY_WORKLOAD] = {
            "value": v2m, "plain_fp64": v2f, "mixed_over_plain": v2m / v2f, "ms_per_step": sm["ms"] / args.steps,
            "newton_iterations": sm["newton"], "same_newton_iterations": sm["newton"] == sf["newton"],
            "linear_iterations": sm["linear"], "solver_config": {"mixed": sm["cfg"], "fp64": sf["cfg"]},
            "roofline": {"achieved": a2, "frac": a2 / peak, "unit": "GB/s", "peak_kind": peak_kind}}
        for name in ("mixed", "fp64"):
            sec[name]["ctx"].close()
    if not args.headline_only:
        line["lens-48x32"] = lens_line(torch)
        line["lens-vcfv-48x32"] = lens_line(torch, vcfv=True)
        line["blackoil-vcfv-40x20"] = lens_line(torch, blackoil=True)
        line["ensemble-64"] = ensemble_leg(64, torch)
    if world == 1 and not args.no_cpu_baseline:
        v, dt, threads = cpu_sample(prob, iters=1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "Newton iteration 1 of time step 1 of the workload (linearize + "
                                          "BiCGStab/ILU0 to 1e-6 + update; %.1f s)" % dt}
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
    # the plain FP64 form of the same batch (all systems, one untimed run
    # after its autotuner, then one timed run)
    B64 = Batch(probs, params(capi.PREC_FP64))
    B64.autotune(ENSEMBLE["dt"])
    for c in B64.systems:
        c.save_state()
    ext64 = torch.cuda.ExternalStream(B64.stream())

    def one_run64():
        for c in B64.systems:
            c.restore_state()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext64)
        st = B64.time_integration(ENSEMBLE["steps"], ENSEMBLE["dt"])
        e1.record(ext64)
        e1.synchronize()
        if st:
            raise RuntimeError("batched FP64 run failed %d" % st)
        cits = sum(int(B64.report(i)[2].sum()) * int(Ns[i]) for i in range(len(probs)))
        return e0.elapsed_time(e1), cits

    one_run64()
    ms64, cits64 = one_run64()
    batched_fp64 = cits64 / (ms64 / 1000.0)
    same_newton_fp64 = all(B64.report(i)[2].tolist() == newton[i] for i in range(len(probs)))
    B64.close()

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
        "batched_plain_fp64": {"value": batched_fp64, "same_newton_iterations": same_newton_fp64},
        "batched_over_one_at_a_time": (value / world) / one_value,
        "batched_mixed_over_plain_fp64": (value / world) / one_fp64,
        "batched_mixed_over_batched_plain_fp64": (value / world) / batched_fp64,
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


# Served stream: the configured Poisson rates (50-2000 req/s) all exceed what
# one GPU serves at these sizes (saturated server, latency = queueing), so
# unsaturated rates (0.25 and 1 req/s) are measured beside them, where
# latency shows the service time; requests per rate as given in `requests`
SERVE = dict(lo=20000, hi=1000000, pool=12, rates=(0.25, 1.0, 50, 2000),
             requests={0.25: 100, 1.0: 200, 50: 200, 2000: 200}, baseline_requests=24, seed=2024,
             dt=86400.0, capacity=16, cluster=8, lanes=((150000, 12, 4),))


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

    def trace(rate, seed, count=None):
        r = np.random.default_rng(seed)
        n = count if count is not None else SERVE["requests"][rate]
        t = np.cumsum(r.exponential(1.0 / rate, n))
        return [Request(probs[i % len(probs)], steps=1, dt=SERVE["dt"], arrival=float(a), rid=i)
                for i, a in enumerate(t)]

    def seed_of(rate):
        return int(round(rate * 1000))

    # one lane: every request in one batch
    srv = Server(capi.MODEL_BLACKOIL_3P, prm, capacity=SERVE["capacity"], cluster_size=SERVE["cluster"],
                 max_cells=big)
    serve(srv, trace(1000, 1, 4))  # warm-up: module load, graphs, pinned buffers
    top_rate = SERVE["rates"][-1]
    single = latency_summary(serve(srv, trace(top_rate, seed_of(top_rate))))
    srv.close()
    # size lanes: requests up to 150k cells in clusters of 4, larger ones in
    # clusters of 16, side by side on their own streams
    laned = LanedServer(capi.MODEL_BLACKOIL_3P, prm, lanes=SERVE["lanes"] + ((big, 4, 16),))
    serve_laned(laned, trace(1000, 1, 6))
    sampler = ClockSampler(0)
    sampler.start()
    served = {}
    for rate in SERVE["rates"]:
        reqs = serve_laned(laned, trace(rate, seed_of(rate)))
        served[str(rate)] = latency_summary(reqs)
    clocks = sampler.stop()
    laned.close()
    base = {}
    for rate in (SERVE["rates"][1], SERVE["rates"][-1]):
        reqs = serve_one_at_a_time(trace(rate, seed_of(rate), SERVE["baseline_requests"]), params(capi.PREC_FP64))
        base[str(rate)] = latency_summary(reqs)
    top = str(SERVE["rates"][-1])
    line = {
        "metric": METRIC, "value": served[top]["cell_newton_its_per_s"], "unit": UNIT, "n_gpus": 1,
        "steps": len(SERVE["rates"]), "warmup": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 residual/Jacobian/update + f32 ILU0/BiCGStab",
        "data": "synthetic (seeded black-oil grids, cells log-uniform 20k-1M, lognormal permeability sigma 1)",
        "config": {"workload": "served stream of single-time-step black-oil solves, Poisson arrivals at %s req/s "
                               "(%s requests), continuous batching, admission by HBM footprint, "
                               "mixed precision" % (list(SERVE["rates"]), [SERVE["requests"][r] for r in SERVE["rates"]]),
                   "pool_cells": [int(p.num_cells) for p in probs],
                   "lanes": "cells <= 150k: 12 slots, clusters of 4; larger: 4 slots, clusters of 16",
                   "parallelism": "single GPU"},
        "served": served,
        "one_lane_at_top_rate": single,
        "one_at_a_time_fp64": base,
        "throughput_vs_offered": [[served[str(r)]["offered_rps"], served[str(r)]["throughput_rps"]]
                                  for r in SERVE["rates"]],
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
