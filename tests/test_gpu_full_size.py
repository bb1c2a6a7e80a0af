"""Parity at the benchmark's full size (the 100x100x20 black-oil workload,
200k cells, 10 one-day steps, BiCGStab + ILU(0) to 1e-6, Newton tolerance
1e-6) against the oracle's log of the same run (tests/golden/
blackoil_100x100x20_newton_log.npz, made by
tests/golden/make_blackoil_100x100x20_golden.py).  Both the FP64
and the mixed-precision run have the oracle's Newton counts per step and its
meanings at sampled cells; the FP64 run's total of linear iterations is
within 10 % (the dot products sum in another order, and single BiCGStab
solves near their tolerance move by up to ~20 % with it).  The states agree
to what the benchmark's tolerances leave (STATE_RTOL_BENCH: two correct
solvers' solutions of a system solved to 1e-6 differ at that level, and so
do the mixed-precision and FP64 runs; a Newton tolerance of 1e-6 on the
residual leaves pressures free by kPa at this compressibility), and the
GPU's final state is converged by the oracle's own residual: the oracle,
given the GPU's states before and after the last step, finds a Newton error
within the Newton tolerance.  With tight solves (linear 1e-10, Newton 1e-8,
two steps, blackoil_100x100x20_tight_log.npz) the FP64 state agrees to
STATE_RTOL_TIGHT."""
import os

import numpy as np
import pytest

import oracle as O

from gbfv import Context, capi, problems
from parity import rel_state_diff

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blackoil_100x100x20_newton_log.npz")
TIGHT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blackoil_100x100x20_tight_log.npz")
STATE_RTOL_BENCH = 1e-4
STATE_RTOL_TIGHT = 1e-6


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_blackoil_100x100x20_against_the_oracle_log(built, precision):
    g = np.load(GOLDEN)
    prob = problems.blackoil(100, 100, 20)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=precision,
                              inner_tolerance=1e-6)
    ctx = Context(prob, prm)
    st, dts, nits, lits, _ = ctx.time_integration(9, 86400.0, fixed_dt=True)
    assert st == 0
    x9, m9 = ctx.solution()
    st, rep = ctx.newton_apply(86400.0)
    assert st == 0
    nits = np.append(nits, rep.iterations)
    lits = np.append(lits, rep.linear_iterations)
    x, m = ctx.solution()
    ctx.close()
    assert np.array_equal(nits, g["newton"]), (nits, g["newton"])
    assert np.array_equal(dts, g["dt"][:9])
    # the oracle's residual at the GPU's last step (old level: the GPU's step-9 state)
    orc = O.Oracle(prob, prm)
    orc.set_solution(x9, m9)
    assert orc.linearize(86400.0, 0) == 0
    orc.set_solution(x, m)
    assert orc.linearize(86400.0, 1) == 0
    err = orc.newton_error()
    assert err <= prm.newton_tolerance, err
    idx = g["cells"]
    assert np.array_equal(m[idx], g["meaning"])
    diff = rel_state_diff(x.reshape(-1, 3)[idx].ravel(), g["pv"].ravel(), 3)
    assert diff <= STATE_RTOL_BENCH, diff
    if precision == capi.PREC_FP64:
        assert abs(int(lits.sum()) - int(g["linear"].sum())) <= 0.1 * g["linear"].sum(), (lits, g["linear"])


def test_blackoil_100x100x20_tight_solves_match_the_oracle_state(built):
    g = np.load(TIGHT)
    prob = problems.blackoil(100, 100, 20)
    prm = capi.default_params(linear_tolerance=1e-10, newton_tolerance=1e-8)
    ctx = Context(prob, prm)
    st, dts, nits, lits, _ = ctx.time_integration(len(g["newton"]), 86400.0, fixed_dt=True)
    x, m = ctx.solution()
    ctx.close()
    assert st == 0
    assert np.array_equal(nits, g["newton"]), (nits, g["newton"])
    idx = g["cells"]
    assert np.array_equal(m[idx], g["meaning"])
    assert rel_state_diff(x.reshape(-1, 3)[idx].ravel(), g["pv"].ravel(), 3) <= STATE_RTOL_TIGHT
