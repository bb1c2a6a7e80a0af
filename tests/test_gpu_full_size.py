"""Parity at the benchmark's full size (workload C2: 100x100x20 black-oil,
200k cells, 10 one-day steps, BiCGStab + ILU(0) to 1e-6, Newton tolerance
1e-6) against the oracle's log of the same run (tests/golden/
c2_newton_log.npz, made by tests/golden/make_c2_golden.py): the FP64 run has
the oracle's Newton counts per step, its total of linear iterations within
10 % (the dot products sum in another order, and single BiCGStab solves near
their tolerance move by up to ~20 % with it), and at sampled cells the
oracle's meanings and
primary variables to 1e-8; the mixed-precision run keeps the Newton counts
(its state moves by up to what the 1e-6 linear tolerance leaves, 2e-5 as in
the smaller mixed-precision test)."""
import os

import numpy as np
import pytest

from gbfv import Context, capi, problems
from parity import rel_state_diff

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c2_newton_log.npz")


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_c2_against_the_oracle_log(built, precision):
    g = np.load(GOLDEN)
    prob = problems.blackoil(100, 100, 20)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=precision,
                              inner_tolerance=1e-6)
    ctx = Context(prob, prm)
    st, dts, nits, lits, _ = ctx.time_integration(10, 86400.0, fixed_dt=True)
    x, m = ctx.solution()
    ctx.close()
    assert st == 0
    assert np.array_equal(nits, g["newton"]), (nits, g["newton"])
    assert np.array_equal(dts, g["dt"])
    idx = g["cells"]
    assert np.array_equal(m[idx], g["meaning"])
    diff = rel_state_diff(x.reshape(-1, 3)[idx].ravel(), g["pv"].ravel(), 3)
    if precision == capi.PREC_FP64:
        assert abs(int(lits.sum()) - int(g["linear"].sum())) <= 0.1 * g["linear"].sum(), (lits, g["linear"])
        assert diff <= 1e-8, diff
    else:
        assert diff <= 2e-5, diff
