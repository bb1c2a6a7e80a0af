"""GPU parity of the vertex-centred discretization (problem.num_elements >
0: VcfvDiscretization with P1 or two-point gradients, the lens VCFV tests'
configuration) against the oracle's restatement (oracle/vcfv.hh): the
residual and the 9-point Jacobian at the 1e-12 bar, the general block
ILU(0) to rounding, one solve, Newton through the lens time loop with
ILU(0) and with AMG, the finite-difference linearizer, and what it
refuses."""
import numpy as np
import pytest

import oracle as O
from gbfv import Context, LinearSolver, capi, problems
from parity import RTOL_LIN, jacobian_mismatch_fast, rel_state_diff, residual_mismatch

pytestmark = pytest.mark.gpu


def _prm(**kw):
    kw.setdefault("linear_tolerance", 1e-8)
    return capi.default_params(**kw)


def _perturbed(prob, seed=2):
    rng = np.random.default_rng(seed)
    pv = prob.init_pv.reshape(-1, 2).copy()
    pv[:, 1] = rng.uniform(0.6, 1.0, len(pv))
    pv[:, 0] *= 1.0 + 1e-3 * rng.standard_normal(len(pv))
    return pv.ravel()


def _compare(ctx, orc, dt, it):
    assert ctx.linearize(dt, it) == 0
    assert orc.linearize(dt, it) == 0
    rg, ro, sc = ctx.residual(), orc.residual(), orc.residual_scale()
    rpg, colg, jg = ctx.jacobian()
    rpo, colo, jo = orc.jacobian()
    assert np.array_equal(rpg, rpo) and np.array_equal(colg, colo)
    return residual_mismatch(rg, ro, sc), jacobian_mismatch_fast(rpo, colo, jg, jo)


@pytest.mark.parametrize("p1", [True, False])
def test_linearization_matches_the_oracle(built, p1):
    prob = problems.lens_vcfv(p1=p1)
    ctx = Context(prob, _prm())
    orc = O.Oracle(prob, _prm())
    er, ej = _compare(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)
    pv = _perturbed(prob)
    for it in (1, 2):
        ctx.set_solution(pv, prob.init_meaning)
        orc.set_solution(pv, prob.init_meaning)
        er, ej = _compare(ctx, orc, 250.0, it)
        assert er <= RTOL_LIN and ej <= RTOL_LIN, (it, er, ej)


def test_residual_agrees_to_rounding(built):
    """Values follow the oracle's operation order with FMA contraction off
    on both sides and the elements summed in the same order: what remains
    is the last-ulp difference of the math library's pow in the material
    law."""
    prob = problems.lens_vcfv(12, 8)
    ctx = Context(prob, _prm())
    orc = O.Oracle(prob, _prm())
    pv = _perturbed(prob)
    for o in (ctx, orc):
        o.linearize(250.0, 0)
        o.set_solution(pv, prob.init_meaning)
        o.linearize(250.0, 1)
    assert residual_mismatch(ctx.residual(), orc.residual(), orc.residual_scale()) <= 1e-14


def test_general_ilu0_matches_the_oracle(built):
    """The block ILU(0) of the 9-point Jacobian (lower entries updating the
    whole shared part of the row) applied once, FP64: the oracle's
    blockILU0Decomposition + back-solve in the same order, to rounding (the
    device contracts products to FMAs)."""
    prob = problems.lens_vcfv()
    orc = O.Oracle(prob, _prm())
    assert orc.time_integration(2, 250.0)[0] == 0
    assert orc.linearize(250.0, 0) == 0
    rp, col, blk = orc.jacobian()
    n = len(rp) - 1
    ls = LinearSolver(rp, col, 2, _prm())
    ls.set_matrix(blk)
    rng = np.random.default_rng(4)
    for d in (orc.residual(), rng.standard_normal(2 * n)):
        st, _, vo = O.ilu0(rp, col, blk, d)
        assert st == 0
        vg = ls.ilu0_apply(d)
        assert np.max(np.abs(vg - vo)) <= 1e-13 * np.max(np.abs(vo)), np.max(np.abs(vg - vo))


def test_one_solve_matches_the_oracle(built):
    prob = problems.lens_vcfv()
    prm = _prm()
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    assert orc.time_integration(2, 250.0)[0] == 0
    pv, m = orc.solution()
    ctx.set_solution(pv, m)
    assert orc.linearize(250.0, 0) == 0 and ctx.linearize(250.0, 0) == 0
    rp, col, blk = orc.jacobian()
    so, xo, ito = O.bcrs_solve(rp, col, blk, orc.residual(), prm)
    sg, xg, itg = ctx.solve()
    assert so == 0 and sg == 0
    assert abs(itg - ito) <= 2, (itg, ito)
    assert np.max(np.abs(xg - xo)) <= 1e-6 * np.max(np.abs(xo))


@pytest.mark.parametrize("solver", ["ilu0", "amg"])
def test_lens_time_loop_matches_the_oracle(built, solver):
    """30 lens steps on the vertex-centred grid: the same time steps and
    Newton counts, the state within 1e-8."""
    prob = problems.lens_vcfv()
    kw = dict(linear_tolerance=1e-10)
    if solver == "amg":
        kw.update(linear_solver=capi.LINSOLVER_AMG, amg_coarsen_target=100)
    prm = _prm(**kw)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    so, dto, no, lo, _ = orc.time_integration(30, 250.0)
    sg, dtg, ng, lg, _ = ctx.time_integration(30, 250.0)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    assert np.allclose(dto, dtg, rtol=1e-12, atol=0)
    pvo, _ = orc.solution()
    pvg, _ = ctx.solution()
    assert rel_state_diff(pvg, pvo, 2) <= 1e-8


def test_mixed_precision_meets_the_tolerance(built):
    """FP32 BiCGStab + FP32 general ILU(0) under FP64 refinement reaches the
    FP64 solution to the tolerance's envelope."""
    prob = problems.lens_vcfv()
    ctx64 = Context(prob, _prm())
    ctx = Context(prob, _prm(precision=capi.PREC_MIXED, inner_tolerance=1e-4))
    assert ctx64.time_integration(3, 250.0)[0] == 0
    ctx.set_solution(*ctx64.solution())
    for c in (ctx64, ctx):
        assert c.linearize(250.0, 0) == 0
    s64, x64, _ = ctx64.solve()
    sg, xg, itg = ctx.solve()
    assert s64 == 0 and sg == 0 and itg > 0
    assert np.max(np.abs(xg - x64)) <= 1e-6 * np.max(np.abs(x64))


@pytest.mark.parametrize("method", [1, 0, -1])
def test_fd_linearization_matches_the_oracle(built, method):
    """The finite-difference local linearizer (lens_immiscible_vcfv_fd):
    residual at 1e-12; the difference quotients at 1e-5 on the initial state
    and 1e-3 on a randomly perturbed one -- the two sides' residuals differ
    by rounding (the math library's pow in the material law, here up to
    5e-14 of the summed terms), which the quotient divides by eps ~ 1e-10."""
    prob = problems.lens_vcfv()
    prm = _prm(local_linearizer=capi.LIN_FD, numeric_difference_method=method)
    ctx = Context(prob, prm)
    orc = O.Oracle(prob, prm)
    er, ej = _compare(ctx, orc, 250.0, 0)
    assert er <= RTOL_LIN and ej <= 1e-5, (er, ej)
    pv = _perturbed(prob)
    ctx.set_solution(pv, prob.init_meaning)
    orc.set_solution(pv, prob.init_meaning)
    er, ej = _compare(ctx, orc, 250.0, 1)
    assert er <= RTOL_LIN and ej <= 1e-3, (er, ej)


def test_fd_time_loop_matches_the_oracle(built):
    prob = problems.lens_vcfv()
    prm = _prm(local_linearizer=capi.LIN_FD, linear_tolerance=1e-10)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    so, dto, no, lo, _ = orc.time_integration(10, 250.0)
    sg, dtg, ng, lg, _ = ctx.time_integration(10, 250.0)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    pvo, _ = orc.solution()
    pvg, _ = ctx.solution()
    assert rel_state_diff(pvg, pvo, 2) <= 1e-7


def test_refuses_what_it_does_not_model(built):
    with pytest.raises(RuntimeError, match="ERR_UNSUPPORTED"):
        Context(problems.lens_vcfv(6, 4), _prm(linearizer=capi.LINEARIZER_TPFA))
    bad = problems.lens_vcfv(6, 4)
    bad.elem_corner = bad.elem_corner.reshape(-1, 4)[:, [1, 0, 2, 3]].ravel().copy()
    with pytest.raises(RuntimeError, match="ERR_UNSUPPORTED"):
        Context(bad, _prm())
    with pytest.raises(RuntimeError, match="ERR_UNSUPPORTED"):
        from gbfv import Batch
        Batch([problems.lens_vcfv(6, 4)], _prm())


def _bo_state(prob, seed=3):
    rng = np.random.default_rng(seed)
    pv = prob.init_pv.reshape(-1, 3).copy()
    pv[:, 1] *= 1.0 + 0.01 * rng.standard_normal(len(pv))
    pv[:, 0] = rng.uniform(0.1, 0.3, len(pv))
    m = prob.init_meaning.copy()
    m[::3] = capi.GAS_SG
    pv[::3, 2] = rng.uniform(0.0, 0.2, len(pv[::3]))
    return pv.ravel(), m


def test_blackoil_linearization_matches_the_oracle(built):
    """The black-oil model on the vertex-centred stencil (reservoir_blackoil_vcfv):
    residual and Jacobian at 1e-12, with both gas meanings and wells as
    constraint vertices."""
    prob = problems.blackoil_vcfv(20, 10)
    prm = _prm(newton_tolerance=1e-6)
    ctx = Context(prob, prm)
    orc = O.Oracle(prob, prm)
    er, ej = _compare(ctx, orc, 86400.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)
    pv, m = _bo_state(prob)
    for it in (1, 2):
        ctx.set_solution(pv, m)
        orc.set_solution(pv, m)
        er, ej = _compare(ctx, orc, 86400.0, it)
        assert er <= RTOL_LIN and ej <= RTOL_LIN, (it, er, ej)


def test_blackoil_time_loop_matches_the_oracle(built):
    """Five days of the vertex-centred black-oil section with its wells:
    the same Newton counts, the same gas meanings, the state within 1e-8."""
    prob = problems.blackoil_vcfv(20, 10)
    prm = _prm(linear_tolerance=1e-10, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    so, _, no, _, _ = orc.time_integration(5, 86400.0, fixed_dt=True)
    sg, _, ng, _, _ = ctx.time_integration(5, 86400.0, fixed_dt=True)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    pvo, mo = orc.solution()
    pvg, mg = ctx.solution()
    assert np.array_equal(mo, mg)
    assert rel_state_diff(pvg, pvo, 3) <= 1e-8


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_tagged_sweeps_equal_level_sweeps(built, monkeypatch, prec):
    """The general kernel on 8 blocks (the narrow path off): its tagged
    sweeps (rows publish tagged results, no barrier per level) give the
    level-barrier sweeps' solution to the bit, iteration count included."""
    prob = problems.lens_vcfv()
    prm = _prm(precision=prec)
    monkeypatch.setenv("GBFV_GILU_BLOCKS", "8")
    monkeypatch.setenv("GBFV_GILU_WARP", "0")
    out = []
    for tagged in ("0", "1"):
        monkeypatch.setenv("GBFV_GILU_TAGGED", tagged)
        monkeypatch.setenv("GBFV_GILU_TAGGED64", tagged)
        ctx = Context(prob, prm)
        mode = ctx.solver_config(prec)["mode"]
        assert mode == ("gilu+tagged" if tagged == "1" else "gilu"), mode
        assert ctx.linearize(250.0, 0) == 0
        out.append(ctx.solve())
        ctx.close()
    (s0, x0, i0), (s1, x1, i1) = out
    assert s0 == 0 and s1 == 0 and i0 == i1
    assert np.array_equal(x0, x1)
