"""GPU checks of the persistent solver's launch modes: the spatial-tile
sweeps (rows of every ILU level dealt to the cluster's blocks by the tile of
their cell, dependencies across tiles pushed into halo slots) give the same
result as the push sweeps with the same cluster, and agree with the CPU
oracle in FP64, alone and in the hybrid launch."""
import numpy as np
import pytest

import oracle as O
from gbfv import Context, capi, problems
from parity import rel_state_diff

pytestmark = pytest.mark.gpu

TILES = capi.SOLVER_TILES


def _run(prob, prm, prec, mode, blocks, steps, dt):
    ctx = Context(prob, prm)
    ctx.set_solver_config(prec, mode, blocks)
    st, sdt, sn, sl, _ = ctx.time_integration(steps, dt, fixed_dt=True)
    x, m = ctx.solution()
    cfg = ctx.solver_config(prec)
    ctx.close()
    return st, sn, sl, x, m, cfg


@pytest.mark.parametrize("shape", [(32, 28, 6), (9, 7, 3)])
def test_tile_sweeps_equal_push_sweeps(built, shape):
    prob = problems.blackoil(*shape, seed=5)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                              inner_tolerance=1e-5)
    a = _run(prob, prm, capi.PREC_MIXED, capi.SOLVER_CLUSTER, 16, 3, 86400.0)
    b = _run(prob, prm, capi.PREC_MIXED, capi.SOLVER_CLUSTER | TILES, 16, 3, 86400.0)
    assert a[0] == 0 and b[0] == 0
    assert b[5]["mode"] == "cluster+tiles" and b[5]["blocks"] == 16
    # the same arithmetic per row, the same reductions: the same iterates
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), (a[1], b[1], a[2], b[2])
    assert np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])


def test_tile_sweeps_lens_fp64_match_oracle(built):
    prob = problems.lens()
    prm = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    so, dto, no, lo, tlo = orc.time_integration(30, 250.0)
    ctx = Context(prob, prm)
    ctx.set_solver_config(capi.PREC_FP64, capi.SOLVER_CLUSTER | TILES, 16)
    sg, dtg, ng, lg, tlg = ctx.time_integration(30, 250.0)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    assert np.allclose(dto, dtg, rtol=1e-12, atol=0)
    assert rel_state_diff(ctx.solution()[0], orc.solution()[0], 2) <= 1e-8


@pytest.mark.parametrize("mode,blocks", [(capi.SOLVER_CLUSTER | TILES, 16), (capi.SOLVER_HYBRID | TILES, 32)])
def test_tile_sweeps_blackoil_fp64_match_oracle(built, mode, blocks):
    prob = problems.blackoil(24, 20, 6)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    so, _, no, _, _ = orc.time_integration(4, 86400.0, fixed_dt=True)
    sg, ng, lg, x, m, cfg = _run(prob, prm, capi.PREC_FP64, mode, blocks, 4, 86400.0)
    assert so == 0 and sg == 0
    assert cfg["mode"].endswith("+tiles")
    assert np.array_equal(no, ng), (no, ng)
    pvo, mo = orc.solution()
    assert np.array_equal(mo, m)
    assert rel_state_diff(x, pvo, 3) <= 1e-8


def test_hybrid_tiles_mixed_equal_alone_runs(built):
    """Two contexts with the same hybrid+tiles configuration give the same
    bits (the pipeline's timing does not enter the arithmetic)."""
    prob = problems.blackoil(40, 36, 8, seed=9)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                              inner_tolerance=1e-5)
    a = _run(prob, prm, capi.PREC_MIXED, capi.SOLVER_HYBRID | TILES, 32, 2, 86400.0)
    b = _run(prob, prm, capi.PREC_MIXED, capi.SOLVER_HYBRID | TILES, 32, 2, 86400.0)
    assert a[0] == 0 and b[0] == 0
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])


def test_tile_flag_needs_a_cluster_mode(built):
    ctx = Context(problems.blackoil(8, 8, 3), capi.default_params())
    with pytest.raises(Exception):
        ctx.set_solver_config(capi.PREC_FP64, capi.SOLVER_GRID | TILES, 16)
    ctx.close()


def test_narrow_hybrid_mixed_keeps_the_fp64_newton_counts(built):
    """The mixed-precision hybrid launch with 256-thread blocks: the same
    Newton counts as the FP64 run and its state to what the linear
    tolerance leaves, as the 512-thread launch."""
    prob = problems.blackoil(40, 36, 8, seed=9)
    pmx = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                              inner_tolerance=1e-5)
    p64 = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    st, n, _, x, m, cfg = _run(prob, pmx, capi.PREC_MIXED, capi.SOLVER_HYBRID | capi.SOLVER_NARROW, 32, 3,
                               86400.0)
    assert st == 0 and cfg["mode"] == "hybrid-256"
    st, n64, _, x64, m64, _ = _run(prob, p64, capi.PREC_FP64, capi.SOLVER_CLUSTER, 16, 3, 86400.0)
    assert st == 0
    assert np.array_equal(n, n64), (n, n64)
    assert np.array_equal(m, m64)
    assert rel_state_diff(x, x64, 3) <= 2e-5


def _wide_params(prec, tol):
    return capi.default_params(linear_tolerance=tol, newton_tolerance=1e-6, precision=prec, inner_tolerance=1e-6)


def test_tagged_sweeps_equal_the_cluster_sweeps(built, monkeypatch):
    """A system wider than one block of the general kernel (72,000 cells)
    solved with its tagged sweeps (GBFV_SOLVER=tagged: every row publishes
    its result with a tag that its consumers wait for; no barrier per
    wavefront level) against the structured cluster sweeps forced on the
    same system, mixed precision: the FP32 inner solves do the same
    operations, so two time steps give the same Newton and linear iteration
    counts, gas meanings and states."""
    monkeypatch.setenv("GBFV_SOLVER", "tagged")
    prob = problems.blackoil(60, 60, 20, seed=7)
    prm = _wide_params(capi.PREC_MIXED, 1e-6)
    ctx = Context(prob, prm)
    assert ctx.solver_config(capi.PREC_MIXED)["mode"] == "gilu+tagged"
    st, _, sn, sl, _ = ctx.time_integration(2, 86400.0, fixed_dt=True)
    x, m = ctx.solution()
    assert ctx.solver_config(capi.PREC_MIXED)["mode"] == "gilu+tagged"
    ctx.close()
    monkeypatch.delenv("GBFV_SOLVER")
    st2, sn2, sl2, x2, m2, cfg = _run(prob, prm, capi.PREC_MIXED, capi.SOLVER_CLUSTER, 16, 2, 86400.0)
    assert st == 0 and st2 == 0 and cfg["mode"] == "cluster"
    assert np.array_equal(sn, sn2) and np.array_equal(m, m2)
    assert np.abs(np.asarray(sl) - np.asarray(sl2)).max() <= 2, (sl, sl2)
    assert rel_state_diff(x, x2, 3) <= 1e-8


def test_tagged_fp64_solve_matches_the_cluster_solve(built, monkeypatch):
    """The same in FP64 on one linear system (the first Newton iteration of
    the first day, solved to a 1e-10 reduction with no absolute floor): the
    general kernel contracts its products to FMAs and the structured one
    does not, so the two solves differ by rounding.  Both meet the system
    (true max-norm residual of J dx = r within 1e-9 of max |r|, J taken
    from the context), their iteration counts are within 10 % and the
    updates within 1e-5 of their size."""
    sp = pytest.importorskip("scipy.sparse")
    prob = problems.blackoil(60, 60, 20, seed=7)
    prm = capi.default_params(linear_tolerance=1e-10, linear_abs_tolerance=0.0, newton_tolerance=1e-6,
                              precision=capi.PREC_FP64)
    out = []
    for tagged in (True, False):
        if tagged:
            monkeypatch.setenv("GBFV_SOLVER", "tagged")
        else:
            monkeypatch.delenv("GBFV_SOLVER")
        ctx = Context(prob, prm)
        if not tagged:
            ctx.set_solver_config(capi.PREC_FP64, capi.SOLVER_CLUSTER, 16)
        assert ctx.solver_config(capi.PREC_FP64)["mode"] == ("gilu+tagged" if tagged else "cluster")
        assert ctx.linearize(86400.0, 0) == 0
        st, dx, it = ctx.solve()
        r = ctx.residual()
        rp, col, blk = ctx.jacobian()
        J = sp.bsr_matrix((blk, col, rp), shape=(len(r), len(r)))
        out.append((st, dx, it, np.max(np.abs(r - J @ dx)) / np.max(np.abs(r))))
        ctx.close()
    (s0, x0, i0, e0), (s1, x1, i1, e1) = out
    assert s0 == 0 and s1 == 0
    assert e0 <= 1e-9 and e1 <= 1e-9, (e0, e1)
    assert abs(i0 - i1) <= 0.1 * i1, (i0, i1)
    assert np.max(np.abs(x0 - x1)) <= 1e-5 * np.max(np.abs(x1))
