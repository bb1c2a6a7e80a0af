"""GPU finite-difference linearizer (FvBaseFdLocalLinearizer) against the
oracle's: the residual at the 1e-12 bar; the Jacobian, whose entries are
differences of residuals divided by deflections of about 1e-10 (relative),
to FD_RTOL of the largest entry of the same (equation, variable) in the
row -- a last-bit difference of a residual value, as between CUDA's and the
host's pow, shows up there about 1e6 times larger; then Newton runs with
the same iteration counts and states to FD_STATE_RTOL (the Jacobians' small
differences move each Newton update by a little, inside the linear
tolerance, so the states agree less closely than the AD runs' 1e-8)."""
import numpy as np
import pytest

import oracle as O
from gbfv import Context, capi, problems
from parity import RTOL_LIN, jacobian_mismatch_fast, rel_state_diff, residual_mismatch

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-5
FD_STATE_RTOL = 1e-7


def _compare(prob, prm, dt, state):
    ctx, orc = Context(prob, prm), O.Oracle(prob, prm)
    out = []
    for it in (0, 1):
        for o in (ctx, orc):
            o.set_solution(*state)
        for o in (ctx, orc):
            assert o.linearize(dt, it) == 0
        er = residual_mismatch(ctx.residual(), orc.residual(), orc.residual_scale())
        rpg, colg, jg = ctx.jacobian()
        rpo, colo, jo = orc.jacobian()
        assert np.array_equal(rpg, rpo) and np.array_equal(colg, colo)
        out.append((er, jacobian_mismatch_fast(rpo, colo, jg, jo)))
    ctx.close()
    return out


@pytest.mark.parametrize("method", [1, 0, -1])
def test_fd_lens_linearization(built, method):
    prob = problems.lens()
    base = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, base)
    assert orc.time_integration(6, 250.0)[0] == 0
    prm = capi.default_params(linear_tolerance=1e-6, local_linearizer=capi.LIN_FD, numeric_difference_method=method)
    for er, ej in _compare(prob, prm, 300.0, orc.solution()):
        assert er <= RTOL_LIN and ej <= FD_RTOL, (method, er, ej)


@pytest.mark.parametrize("method", [1, 0])
def test_fd_blackoil_linearization(built, method):
    prob = problems.blackoil(9, 7, 4)
    base = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    orc = O.Oracle(prob, base)
    assert orc.time_integration(3, 86400.0, fixed_dt=True)[0] == 0
    state = orc.solution()
    assert (state[1] == capi.GAS_SG).any() and (state[1] == capi.GAS_RS).any()
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, local_linearizer=capi.LIN_FD,
                              numeric_difference_method=method)
    for er, ej in _compare(prob, prm, 86400.0, state):
        assert er <= RTOL_LIN and ej <= FD_RTOL, (method, er, ej)


@pytest.mark.parametrize("kind", ["lens", "blackoil"])
def test_fd_newton_matches_oracle(built, kind):
    if kind == "lens":
        prob, dt, steps = problems.lens(), 250.0, 15
        prm = capi.default_params(linear_tolerance=1e-6, local_linearizer=capi.LIN_FD)
    else:
        prob, dt, steps = problems.blackoil(12, 10, 4), 86400.0, 4
        prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, local_linearizer=capi.LIN_FD)
    orc, ctx = O.Oracle(prob, prm), Context(prob, prm)
    so, dto, no, _, _ = orc.time_integration(steps, dt, fixed_dt=kind == "blackoil")
    sg, dtg, ng, _, _ = ctx.time_integration(steps, dt, fixed_dt=kind == "blackoil")
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    xo, mo = orc.solution()
    xg, mg = ctx.solution()
    assert np.array_equal(mo, mg)
    assert rel_state_diff(xg, xo, prob.b) <= FD_STATE_RTOL
    ctx.close()


def test_fd_not_accepted_by_batches(built):
    from gbfv import Batch
    prm = capi.default_params(local_linearizer=capi.LIN_FD)
    with pytest.raises(Exception):
        Batch([problems.blackoil(6, 5, 3)], prm, cluster_size=2)
