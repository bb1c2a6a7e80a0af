"""GPU parity: linearization, linear solve and Newton of libgbfv against the
CPU oracle on the same inputs (called through the C ABI)."""
import numpy as np
import pytest

import oracle as O
from gbfv import Context, LinearSolver, capi, problems
from parity import RTOL_LIN, jacobian_mismatch_fast, rel_state_diff, residual_mismatch

pytestmark = pytest.mark.gpu


def _pair(prob, **kw):
    prm = capi.default_params(**kw)
    return Context(prob, prm), O.Oracle(prob, prm)


def _compare_linearization(ctx, orc, dt, it, state=None):
    if state is not None:
        ctx.set_solution(*state)
        orc.set_solution(*state)
    assert ctx.linearize(dt, it) == 0
    assert orc.linearize(dt, it) == 0
    rg, ro, sc = ctx.residual(), orc.residual(), orc.residual_scale()
    rpg, colg, jg = ctx.jacobian()
    rpo, colo, jo = orc.jacobian()
    assert np.array_equal(rpg, rpo) and np.array_equal(colg, colo)
    return residual_mismatch(rg, ro, sc), jacobian_mismatch_fast(rpo, colo, jg, jo)


def test_lens_linearization_initial(built):
    ctx, orc = _pair(problems.lens())
    er, ej = _compare_linearization(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)


@pytest.mark.parametrize("law", ["vg", "bc"])
def test_lens_linearization_with_dnapl(built, law):
    prob = problems.lens(law=law)
    prm = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    st, *_ = orc.time_integration(6, 250.0)
    assert st == 0
    state = orc.solution()
    assert state[0].reshape(-1, 2)[:, 1].min() < 0.99  # DNAPL has entered
    ctx = Context(prob, prm)
    for it in (0, 1):
        er, ej = _compare_linearization(ctx, orc, 300.0, it, state)
        assert er <= RTOL_LIN and ej <= RTOL_LIN, (it, er, ej)


@pytest.mark.parametrize("shape", [(3, 3), (4, 2), (7, 5)])
def test_tiny_lens_grids(built, shape):
    prob = problems.lens(nx=shape[0], ny=shape[1])
    ctx, orc = _pair(prob)
    er, ej = _compare_linearization(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN


def test_blackoil_linearization(built):
    prob = problems.blackoil(9, 7, 4)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    er, ej = _compare_linearization(ctx, orc, 86400.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)
    st, *_ = orc.time_integration(3, 86400.0, fixed_dt=True)
    assert st == 0
    state = orc.solution()
    assert (state[1] == capi.GAS_SG).any() and (state[1] == capi.GAS_RS).any()
    for it in (0, 2):
        er, ej = _compare_linearization(ctx, orc, 86400.0, it, state)
        assert er <= RTOL_LIN and ej <= RTOL_LIN, (it, er, ej)


def test_fp64_solve_matches_oracle(built):
    prob = problems.lens()
    prm = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    orc.time_integration(4, 250.0)
    state = orc.solution()
    ctx = Context(prob, prm)
    ctx.set_solution(*state)
    orc.set_solution(*state)
    ctx.linearize(300.0, 0)
    orc.linearize(300.0, 0)
    sg, dxg, itg = ctx.solve()
    so, dxo, ito = orc.solve()
    assert sg == 0 and so == 0
    assert abs(itg - ito) <= 2, (itg, ito)
    rel = np.max(np.abs(dxg - dxo)) / np.max(np.abs(dxo))
    assert rel < 1e-4, rel


def test_standalone_linsolver(built):
    prob = problems.blackoil(8, 6, 3)
    prm = capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    orc.linearize(86400.0, 0)
    rp, col, blk = orc.jacobian()
    rhs = orc.residual()
    so, xo, ito = O.bcrs_solve(rp, col, blk, rhs, prm)
    ls = LinearSolver(rp, col, 3, prm)
    ls.set_matrix(blk)
    sg, xg, itg = ls.solve(rhs)
    assert so == 0 and sg == 0
    assert np.max(np.abs(xg - xo)) <= 1e-6 * np.max(np.abs(xo))


def test_lens_newton_30_steps(built):
    prob = problems.lens()
    prm = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    so, dto, no, lo, tlo = orc.time_integration(30, 250.0)
    sg, dtg, ng, lg, tlg = ctx.time_integration(30, 250.0)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    assert np.allclose(dto, dtg, rtol=1e-12, atol=0)
    pvo, _ = orc.solution()
    pvg, _ = ctx.solution()
    assert rel_state_diff(pvg, pvo, 2) <= 1e-8


def test_blackoil_newton(built):
    prob = problems.blackoil(12, 10, 4)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    so, dto, no, lo, tlo = orc.time_integration(6, 86400.0, fixed_dt=True)
    sg, dtg, ng, lg, tlg = ctx.time_integration(6, 86400.0, fixed_dt=True)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    pvo, mo = orc.solution()
    pvg, mg = ctx.solution()
    assert np.array_equal(mo, mg)
    assert rel_state_diff(pvg, pvo, 3) <= 1e-8


def test_mixed_precision_same_newton(built):
    prob = problems.blackoil(12, 10, 4)
    p64 = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    pmx = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6,
                              precision=capi.PREC_MIXED, inner_tolerance=1e-5)
    c64 = Context(prob, p64)
    cmx = Context(prob, pmx)
    s64, _, n64, _, _ = c64.time_integration(5, 86400.0, fixed_dt=True)
    smx, _, nmx, _, _ = cmx.time_integration(5, 86400.0, fixed_dt=True)
    assert s64 == 0 and smx == 0
    assert np.array_equal(n64, nmx), (n64, nmx)
    a, _ = c64.solution()
    b, _ = cmx.solution()
    # both runs stop at the same Newton tolerance; the states agree to the
    # size the 1e-6 linear tolerance leaves in each update
    assert rel_state_diff(b, a, 3) <= 2e-5


def test_lens_trans_linearization_and_newton(built):
    """Transmissibility flux module (lens_immiscible_ecfv_ad_trans): residual
    and Jacobian at the initial and a later state, then 30 time steps with the
    same Newton counts and final state as the oracle."""
    prob = problems.lens(flux="trans")
    prm = capi.default_params(linear_tolerance=1e-6)
    ctx, orc = _pair(prob, linear_tolerance=1e-6)
    er, ej = _compare_linearization(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)
    stg, _, sng, _, _ = ctx.time_integration(30, 250.0)
    sto, _, sno, _, _ = orc.time_integration(30, 250.0)
    assert stg == sto == 0
    assert np.array_equal(sng, sno)
    xg, _ = ctx.solution()
    xo, _ = orc.solution()
    assert rel_state_diff(xg, xo, 2) <= 1e-8
    # a later state (the oracle's), storage cache rebuilt from it (iteration 0)
    er, ej = _compare_linearization(ctx, orc, 250.0, 0, state=(xo, None))
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)


@pytest.mark.parametrize("flux", ["darcy", "trans"])
def test_lens_3d_linearization_and_steps(built, flux):
    """3D lens (16x10x6), both flux modules: linearization at the initial
    state, then 6 time steps with the oracle's Newton counts and state."""
    prob = problems.lens(nx=16, ny=10, dim=3, nz=6, flux=flux)
    ctx, orc = _pair(prob, linear_tolerance=1e-8)
    er, ej = _compare_linearization(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)
    stg, _, sng, _, _ = ctx.time_integration(6, 250.0)
    sto, _, sno, _, _ = orc.time_integration(6, 250.0)
    assert stg == sto == 0 and np.array_equal(sng, sno)
    assert rel_state_diff(ctx.solution()[0], orc.solution()[0], 2) <= 1e-8


def test_blackoil_primary_variable_switching_happens(built):
    """The black-oil runs exercise switching: gas appears near the producer
    (Rs -> Sg) and the GPU switches the same cells as the oracle."""
    prob = problems.blackoil(12, 10, 4)
    prm = capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-7)
    ctx, orc = _pair(prob, linear_tolerance=1e-8, newton_tolerance=1e-7)
    m0 = ctx.solution()[1].copy()
    assert ctx.time_integration(4, 86400.0, fixed_dt=True)[0] == 0
    assert orc.time_integration(4, 86400.0, fixed_dt=True)[0] == 0
    xg, mg = ctx.solution()
    xo, mo = orc.solution()
    assert np.array_equal(mg, mo)
    assert int((mg != m0).sum()) > 0, "no primary-variable switch happened"
    assert rel_state_diff(xg, xo, 3) <= 1e-8


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 1, 5), (5, 1, 1), (2, 1, 3), (1, 4, 1)])
def test_degenerate_blackoil_grids(built, shape):
    """Single cells, single rows and columns (both wells in one cell for
    1x1x1): the linearization at the 1e-12 bar, two steps with the oracle's
    Newton counts and state."""
    prob = problems.blackoil(*shape)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    ctx, orc = Context(prob, prm), O.Oracle(prob, prm)
    er, ej = _compare_linearization(ctx, orc, 86400.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (shape, er, ej)
    ctx.close()
    ctx, orc = Context(prob, prm), O.Oracle(prob, prm)
    so, _, no, _, _ = orc.time_integration(2, 86400.0, fixed_dt=True)
    sg, _, ng, _, _ = ctx.time_integration(2, 86400.0, fixed_dt=True)
    assert so == 0 and sg == 0 and np.array_equal(no, ng), (shape, no, ng)
    assert rel_state_diff(ctx.solution()[0], orc.solution()[0], 3) <= 1e-8
    ctx.close()


@pytest.mark.parametrize("shape", [(1, 5), (5, 1), (1, 1), (2, 2)])
def test_degenerate_lens_grids(built, shape):
    prob = problems.lens(nx=shape[0], ny=shape[1])
    prm = capi.default_params(linear_tolerance=1e-6)
    ctx, orc = Context(prob, prm), O.Oracle(prob, prm)
    er, ej = _compare_linearization(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (shape, er, ej)
    ctx.close()
    ctx, orc = Context(prob, prm), O.Oracle(prob, prm)
    so, dto, no, _, _ = orc.time_integration(2, 250.0)
    sg, dtg, ng, _, _ = ctx.time_integration(2, 250.0)
    assert so == 0 and sg == 0 and np.array_equal(no, ng), (shape, no, ng)
    assert rel_state_diff(ctx.solution()[0], orc.solution()[0], 2) <= 1e-8
    ctx.close()
