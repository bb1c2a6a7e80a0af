"""GPU parity of the AMG backend (linear_solver = LINSOLVER_AMG, the
reference's ParallelAmgBackend) against the oracle's restatement
(oracle/amg.hh): the hierarchy, one V-cycle, the preconditioned BiCGStab
solve in FP64 and in mixed precision, and Newton through a context."""
import numpy as np
import pytest

import oracle as O
from gbfv import Context, LinearSolver, capi, problems

pytestmark = pytest.mark.gpu


def _system(prob, dt):
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    o = O.Oracle(prob, prm)
    o.linearize(dt, 0)
    rp, col, blk = o.jacobian()
    return rp, col, blk, o.residual()


CASES = {
    "blackoil-20x16x6": (lambda: problems.blackoil(20, 16, 6), 86400.0, 200),
    "lens-48x32": (lambda: problems.lens(), 250.0, 100),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    mk, dt, target = CASES[request.param]
    rp, col, blk, r = _system(mk(), dt)
    return rp, col, blk, r, target


def _solver(rp, col, blk, target, **kw):
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, linear_solver=capi.LINSOLVER_AMG,
                              amg_coarsen_target=target, **kw)
    ls = LinearSolver(rp, col, blk.shape[-1], prm)
    ls.set_matrix(blk)
    return ls


def test_hierarchy_matches_the_oracle(built, case):
    rp, col, blk, r, target = case
    L, sizes, agg, colors, _ = O.amg(rp, col, blk, target)
    ls = _solver(rp, col, blk, target)
    gs, gc = ls.amg_levels()
    assert L >= 2
    assert np.array_equal(gs, sizes)
    assert gc[0] == colors.max() + 1


def test_one_vcycle_matches_the_oracle(built, case):
    """One FP64 V-cycle: same aggregates, Galerkin sums, colour order,
    operation order and no FMA contraction on both sides, so the results
    agree to the last bit."""
    rp, col, blk, r, target = case
    n, b = len(rp) - 1, blk.shape[-1]
    rng = np.random.default_rng(11)
    ls = _solver(rp, col, blk, target)
    for d in (r, rng.standard_normal(n * b)):
        *_, vo = O.amg(rp, col, blk, target, d)
        vg = ls.amg_apply(d)
        assert np.max(np.abs(vg - vo)) <= 1e-15 * np.max(np.abs(vo)), np.max(np.abs(vg - vo))


def test_fp64_solve_matches_the_oracle(built, case):
    """BiCGStab + AMG in FP64: the iteration count within one of the
    oracle's (the scalar products sum in another order) and the solution
    within the solver tolerance's envelope."""
    rp, col, blk, r, target = case
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, linear_solver=capi.LINSOLVER_AMG,
                              amg_coarsen_target=target)
    so, xo, ito = O.bcrs_solve(rp, col, blk, r, prm)
    ls = _solver(rp, col, blk, target)
    sg, xg, itg = ls.solve(r)
    assert so == 0 and sg == 0
    assert abs(itg - ito) <= 1, (itg, ito)
    assert np.max(np.abs(xg - xo)) <= 1e-5 * np.max(np.abs(xo))


def test_mixed_solve_meets_the_tolerance(built, case):
    """FP32 BiCGStab + FP32 V-cycle under FP64 refinement: the FP64 residual
    of the result meets the relative tolerance, the solution is the FP64
    one to the tolerance's envelope."""
    rp, col, blk, r, target = case
    ls64 = _solver(rp, col, blk, target)
    s64, x64, _ = ls64.solve(r)
    ls = _solver(rp, col, blk, target, precision=capi.PREC_MIXED, inner_tolerance=1e-6)
    sg, xg, itg = ls.solve(r)
    assert s64 == 0 and sg == 0 and itg > 0
    n, b = len(rp) - 1, blk.shape[-1]
    X = xg.reshape(n, b)
    res = r.reshape(n, b).copy()
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            res[i] -= blk[k] @ X[col[k]]
    assert np.max(np.abs(res)) <= 1e-6 * np.max(np.abs(r)) * 1.01
    assert np.max(np.abs(xg - x64)) <= 1e-4 * np.max(np.abs(x64))


def test_lens_newton_through_amg_matches_the_oracle(built):
    """The lens time loop with the AMG backend on both sides: the same
    time steps and Newton counts, the state within 1e-8."""
    prob = problems.lens()
    prm = capi.default_params(linear_tolerance=1e-8, linear_solver=capi.LINSOLVER_AMG, amg_coarsen_target=100)
    orc = O.Oracle(prob, prm)
    ctx = Context(prob, prm)
    so, dto, no, lo, _ = orc.time_integration(10, 250.0)
    sg, dtg, ng, lg, _ = ctx.time_integration(10, 250.0)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    assert np.allclose(dto, dtg, rtol=1e-12, atol=0)
    pvo, _ = orc.solution()
    pvg, _ = ctx.solution()
    scale = np.abs(pvo.reshape(-1, 2)).max(axis=0)
    assert np.max(np.abs((pvg - pvo).reshape(-1, 2)) / scale) <= 1e-8


def test_blackoil_amg_needs_fewer_krylov_iterations(built):
    """On a 50k-cell black-oil system the AMG backend converges in well
    under half the BiCGStab iterations of ILU(0), to the same solution."""
    prob = problems.blackoil(50, 50, 20)
    its, xs = [], []
    for ls_kind in (capi.LINSOLVER_ILU0, capi.LINSOLVER_AMG):
        prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, linear_solver=ls_kind)
        ctx = Context(prob, prm)
        assert ctx.linearize(86400.0, 0) == 0
        st, dx, it = ctx.solve()
        assert st == 0
        its.append(it)
        xs.append(dx)
    assert its[1] * 2 < its[0], its
    assert np.max(np.abs(xs[1] - xs[0])) <= 1e-3 * np.max(np.abs(xs[0]))


def test_single_level_hierarchy_matches_the_oracle(built):
    """A coarsening target at or above the row count leaves one level: the
    V-cycle is the coarsest level's sweeps alone, still equal to the
    oracle's to the last bit, and the solve still converges."""
    rp, col, blk, r = _system(problems.blackoil(8, 6, 3), 86400.0)
    n = len(rp) - 1
    L, sizes, *_ , vo = O.amg(rp, col, blk, n, r)
    assert L == 1
    ls = _solver(rp, col, blk, n)
    gs, gc = ls.amg_levels()
    assert list(gs) == [n]
    vg = ls.amg_apply(r)
    assert np.max(np.abs(vg - vo)) <= 1e-15 * np.max(np.abs(vo))
    sg, xg, itg = ls.solve(r)
    assert sg == 0 and itg > 0


def test_singular_diagonal_block_is_reported(built):
    """A zero diagonal block on some level makes the AMG set-up report
    GBFV_ERR_SINGULAR (the oracle's restatement refuses the same matrix),
    not a silent NaN."""
    rp, col, blk, r = _system(problems.blackoil(6, 5, 3), 86400.0)
    blk = blk.copy()
    n = len(rp) - 1
    for k in range(rp[0], rp[1]):
        if col[k] == 0:
            blk[k][:] = 0.0
    L, *_ = O.amg(rp, col, blk, 200)
    assert L < 0 and -L == capi.ERR_SINGULAR
    ls = _solver(rp, col, blk, 200)
    sg, _, _ = ls.solve(r)
    assert sg == capi.ERR_SINGULAR
