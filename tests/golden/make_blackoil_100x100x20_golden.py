"""Generate the full-size fixture blackoil_100x100x20_newton_log.npz with
the oracle.

Workload blackoil-100x100x20 (200k cells, 10 time steps of one day,
BiCGStab + ILU(0) to 1e-6, Newton tolerance 1e-6, FP64): the oracle's
Newton and linear iteration counts per step, and the final primary
variables of every 997th cell (natural order) with their meanings.  The GPU
test (tests/test_gpu_full_size.py) reruns the workload and compares.
A second log, blackoil_100x100x20_tight_log.npz, is the first two steps
with tight solves (linear tolerance 1e-10, Newton tolerance 1e-8): with the
benchmark's 1e-6
the linear solutions of two correct solvers (different summation orders)
differ by what that tolerance leaves, and the states by ~1e-5; with tight
solves they agree to 1e-8.
Run from the repository root (a few minutes on the host cores each):
    python tests/golden/make_blackoil_100x100x20_golden.py [tight]
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

STRIDE = 997


def main(tight=False):
    prob = problems.blackoil(100, 100, 20)
    if tight:
        prm = capi.default_params(linear_tolerance=1e-10, newton_tolerance=1e-8)
        steps, name = 2, "blackoil_100x100x20_tight_log.npz"
    else:
        prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
        steps, name = 10, "blackoil_100x100x20_newton_log.npz"
    O.set_threads(os.cpu_count() or 1)
    orc = O.Oracle(prob, prm)
    t0 = time.time()
    st, dts, nits, lits, _ = orc.time_integration(steps, 86400.0, fixed_dt=True)
    assert st == 0
    x, m = orc.solution()
    idx = np.arange(0, prob.num_cells, STRIDE)
    np.savez_compressed(os.path.join(HERE, name), newton=nits, linear=lits, dt=dts,
                        cells=idx, pv=x.reshape(-1, 3)[idx], meaning=m[idx])
    print(name, "newton", nits.tolist(), "linear", lits.tolist(), "%.0f s" % (time.time() - t0))


if __name__ == "__main__":
    main(tight=len(sys.argv) > 1 and sys.argv[1] == "tight")
