"""Generate the full-size fixtures (Newton logs and sampled final states)
with the oracle.

Cases (the file each writes):
  c2          blackoil_100x100x20_newton_log.npz   -- the benchmark workload
              (100x100x20 black-oil, 200k cells, 10 one-day steps,
              BiCGStab + ILU(0) to 1e-6, Newton tolerance 1e-6, FP64)
  c2_order    blackoil_100x100x20_dotorder_log.npz -- the same run with the
              BiCGStab scalar products summed in another correct order
              (28672 strided partial sums combined pairwise, as a parallel
              machine sums); nothing else changes.  The gap between c2 and
              c2_order is what summation order alone does to the state at
              these tolerances.
  c2_tight    blackoil_100x100x20_tight_log.npz    -- first two steps, linear
              tolerance 1e-10, Newton tolerance 1e-8
  c2_tight12  blackoil_100x100x20_tight12_log.npz  -- first two steps, linear
              tolerance 1e-12, Newton tolerance 1e-10
  c3          blackoil_100x100x100_newton_log.npz  -- 100x100x100 black-oil
              (1M cells), first two one-day steps, bench tolerances
  c2_amg      blackoil_100x100x20_amg_log.npz      -- 100x100x20, first two
              steps through the AMG backend (linear_solver AMG, coarsening
              target 5000), bench tolerances
  c4member    ensemble_member_largest_log.npz      -- the largest member of
              the 256-realization two-phase ensemble (seeded as the
              benchmark builds it), two steps of 250 s, bench tolerances
Each file holds the oracle's Newton and linear iteration counts and dt per
step, and the final primary variables (and black-oil meanings) of every
STRIDE-th cell in natural order.  The GPU tests (tests/test_gpu_full_size.py)
rerun the case and compare.
Run from the repository root (minutes each on the host cores):
    python tests/golden/make_full_size_golden.py c2 [c2_order ...]
"""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "opm-models_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from gbfv import capi, problems  # noqa: E402

DOT_LANES = 28672  # 112 blocks x 256 threads
ENSEMBLE_SEED, ENSEMBLE_SIZE = 1000, 256


def largest_ensemble_member():
    """The largest of the benchmark's seeded 256 realizations: cell counts
    uniform in [10k, 200k], sigma uniform in [0.5, 1.5], member i seeded
    1000 + i (the order bench.py draws them in)."""
    rng = np.random.default_rng(ENSEMBLE_SEED)
    sizes = rng.integers(10000, 200000 + 1, ENSEMBLE_SIZE)
    sig = rng.uniform(0.5, 1.5, ENSEMBLE_SIZE)
    i = int(np.argmax(sizes))
    return problems.ensemble_member(int(sizes[i]), ENSEMBLE_SEED + i, float(sig[i])), i


def case(name):
    """(problem, params, steps, dt, stride, file name, dot lanes)"""
    bench = dict(linear_tolerance=1e-6, newton_tolerance=1e-6)
    if name == "c2":
        return problems.blackoil(100, 100, 20), bench, 10, 86400.0, 997, "blackoil_100x100x20_newton_log.npz", 0
    if name == "c2_order":
        return (problems.blackoil(100, 100, 20), bench, 10, 86400.0, 997, "blackoil_100x100x20_dotorder_log.npz",
                DOT_LANES)
    if name == "c2_tight":
        return (problems.blackoil(100, 100, 20), dict(linear_tolerance=1e-10, newton_tolerance=1e-8), 2, 86400.0,
                997, "blackoil_100x100x20_tight_log.npz", 0)
    if name == "c2_tight12":
        return (problems.blackoil(100, 100, 20), dict(linear_tolerance=1e-12, newton_tolerance=1e-10), 2, 86400.0,
                997, "blackoil_100x100x20_tight12_log.npz", 0)
    if name == "c3":
        return problems.blackoil(100, 100, 100), bench, 2, 86400.0, 4999, "blackoil_100x100x100_newton_log.npz", 0
    if name == "c2_amg":
        return (problems.blackoil(100, 100, 20), dict(bench, linear_solver=capi.LINSOLVER_AMG), 2, 86400.0, 997,
                "blackoil_100x100x20_amg_log.npz", 0)
    if name == "c4member":
        prob, _ = largest_ensemble_member()
        return prob, bench, 2, 250.0, 997, "ensemble_member_largest_log.npz", 0
    raise SystemExit("unknown case " + name)


def main(name):
    prob, tol, steps, dt, stride, fname, lanes = case(name)
    prm = capi.default_params(**tol)
    O.set_threads(os.cpu_count() or 1)
    O.set_dot_lanes(lanes)
    orc = O.Oracle(prob, prm)
    t0 = time.time()
    st, dts, nits, lits, _ = orc.time_integration(steps, dt, fixed_dt=True)
    assert st == 0, st
    x, m = orc.solution()
    b = len(x) // prob.num_cells
    idx = np.arange(0, prob.num_cells, stride)
    np.savez_compressed(os.path.join(HERE, fname), newton=nits, linear=lits, dt=dts, cells=idx,
                        pv=x.reshape(-1, b)[idx], meaning=m[idx], dot_lanes=lanes)
    print(fname, "newton", nits.tolist(), "linear", lits.tolist(), "%.0f s" % (time.time() - t0))


if __name__ == "__main__":
    for n in sys.argv[1:] or ["c2"]:
        main(n)
