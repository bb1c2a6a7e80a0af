"""Failure detection on the GPU without a fault: a device-side wait that
nothing completes gives up after its bound and reports GBFV_ERR_TIMEOUT; the
device stays usable for the next solve."""
import ctypes as C

import pytest

from gbfv import Context, capi, problems

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_device_stays_usable(built):
    lib = capi.load()
    ms = C.c_double()
    st = lib.gbfv_selftest_wait_timeout(C.byref(ms))
    assert st == capi.ERR_TIMEOUT
    assert 0.0 < ms.value < 5000.0
    ctx = Context(problems.lens(nx=12, ny=8), capi.default_params(linear_tolerance=1e-6))
    rep_st, *_ = ctx.time_integration(2, 250.0)
    assert rep_st == 0


# ---- host-side injection: a bad input comes back as a status code, as in
# the oracle (NumericalProblem -> failed Newton -> dt halving, fvbaseproblem.hh:512-557)

def test_nan_in_state_is_reported_like_the_oracle(built):
    import numpy as np

    import oracle as O
    from gbfv import Context, capi, problems
    prob = problems.blackoil(6, 5, 3)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    x, m = prob.init_pv.copy(), prob.init_meaning.copy()
    x[3 * 7 + 1] = np.nan  # the pressure of one cell
    ctx, orc = Context(prob, prm), O.Oracle(prob, prm)
    for o in (ctx, orc):
        o.set_solution(x, m)
    so, dto, no, lo, _ = orc.time_integration(2, 86400.0)
    sg, dtg, ng, lg, _ = ctx.time_integration(2, 86400.0)
    assert so != 0 and sg == so, (so, sg)
    assert np.array_equal(no, ng) and np.array_equal(dto, dtg)
    ctx.close()
    # the device is fine afterwards: a clean context solves
    ok = Context(prob, prm)
    assert ok.time_integration(1, 86400.0, fixed_dt=True)[0] == 0
    ok.close()


def test_singular_pivot_block_is_reported_like_the_oracle(built):
    import numpy as np

    import oracle as O
    from gbfv import LinearSolver, capi, problems
    prob = problems.blackoil(4, 3, 2)
    prm = capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    assert orc.linearize(86400.0, 0) == 0
    rp, col, blk = orc.jacobian()
    blk = blk.copy()
    c = 5
    k = [j for j in range(rp[c], rp[c + 1]) if col[j] == c][0]
    blk[k] = 0.0  # a zero diagonal block: its ILU(0) pivot cannot be inverted
    rhs = orc.residual()
    so, _, _ = O.bcrs_solve(rp, col, blk, rhs, prm)
    ls = LinearSolver(rp, col, 3, prm)
    ls.set_matrix(blk)
    sg, _, _ = ls.solve(rhs)
    assert so == capi.ERR_SINGULAR and sg == capi.ERR_SINGULAR, (so, sg)


def test_served_request_that_fails_leaves_the_others_unchanged(built):
    import numpy as np

    from gbfv import Context, capi, problems
    from gbfv.serving import Request, Server, serve
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                              inner_tolerance=1e-5)
    good = [problems.blackoil(10, 9, 3, seed=41), problems.blackoil(12, 8, 4, seed=42)]
    bad = problems.blackoil(9, 9, 3, seed=43)
    bad.init_pv = bad.init_pv.copy()
    bad.init_pv[3 * 10 + 1] = np.nan
    reqs = [Request(good[0], steps=1, rid=0), Request(bad, steps=1, rid=1), Request(good[1], steps=1, rid=2)]
    srv = Server(capi.MODEL_BLACKOIL_3P, prm, capacity=3, cluster_size=2, max_cells=4096)
    serve(srv, reqs)
    srv.close()
    assert reqs[1].status != 0
    for r, p in ((reqs[0], good[0]), (reqs[2], good[1])):
        assert r.status == 0
        ctx = Context(p, prm)
        ctx.set_solver_config(capi.PREC_MIXED, 1, 2)
        assert ctx.time_integration(1, 86400.0, fixed_dt=True)[0] == 0
        x, m = ctx.solution()
        ctx.close()
        assert np.array_equal(r.solution[0], x) and np.array_equal(r.solution[1], m)


def test_unknown_gas_meaning_is_rejected_and_the_context_stays_usable(built):
    import numpy as np

    from gbfv import Context, capi, problems
    prob = problems.blackoil(6, 5, 3)
    ctx = Context(prob, capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6))
    bad = np.array(prob.init_meaning, np.int32, copy=True)
    bad[7] = 3  # GasMeaning::Disabled: not a state of this model
    with pytest.raises(Exception):
        ctx.set_solution(prob.init_pv, bad)
    ctx.set_solution(prob.init_pv, prob.init_meaning)
    assert ctx.time_integration(1, 86400.0, fixed_dt=True)[0] == 0
    ctx.close()
