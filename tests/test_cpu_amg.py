"""CPU checks of the AMG restatement (the ParallelAmgBackend path of the
oracle): the hierarchy's structure, the V-cycle as a linear operator, and
BiCGStab + AMG against BiCGStab + ILU(0) on the same systems.  The GPU form
is compared with these in tests/test_gpu_amg.py."""
import numpy as np
import pytest

import oracle as O
from gbfv import capi, problems


def _system(prob, dt):
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    o = O.Oracle(prob, prm)
    o.linearize(dt, 0)
    rp, col, blk = o.jacobian()
    return rp, col, blk, o.residual()


@pytest.fixture(scope="module")
def blackoil_system():
    return _system(problems.blackoil(20, 16, 6), 86400.0)


def _spmv(rp, col, blk, x, b):
    n = len(rp) - 1
    y = np.zeros(n * b)
    X = x.reshape(n, b)
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            y[i * b:(i + 1) * b] += blk[k] @ X[col[k]]
    return y


def test_hierarchy_structure(blackoil_system):
    rp, col, blk, r = blackoil_system
    n = len(rp) - 1
    L, sizes, agg, colors, _ = O.amg(rp, col, blk, coarsen_target=200)
    assert L >= 2 and sizes[0] == n
    assert np.all(np.diff(sizes) < 0) and sizes[-1] <= 200 or L == 15
    # every row in exactly one aggregate, aggregates numbered 0..n1-1, none empty
    assert agg.min() == 0 and agg.max() == sizes[1] - 1
    assert len(np.unique(agg)) == sizes[1]
    # the colouring is proper: no off-diagonal entry joins two rows of one colour
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            if col[k] != i:
                assert colors[col[k]] != colors[i]
    # greedy colouring of a 7-point pattern in natural order is red-black
    assert colors.max() == 1


def test_coarsen_target_stops_coarsening(blackoil_system):
    rp, col, blk, r = blackoil_system
    n = len(rp) - 1
    L, sizes, *_ = O.amg(rp, col, blk, coarsen_target=n)
    assert L == 1 and sizes[0] == n
    L2, sizes2, *_ = O.amg(rp, col, blk, coarsen_target=500)
    assert sizes2[-1] <= 500 and sizes2[-2] > 500


def test_vcycle_is_linear(blackoil_system):
    rp, col, blk, r = blackoil_system
    n = len(rp) - 1
    rng = np.random.default_rng(3)
    d1, d2 = rng.standard_normal(n * 3), rng.standard_normal(n * 3)
    *_, v1 = O.amg(rp, col, blk, 200, d1)
    *_, v2 = O.amg(rp, col, blk, 200, d2)
    *_, v12 = O.amg(rp, col, blk, 200, 2.5 * d1 + d2)
    assert np.max(np.abs(v12 - (2.5 * v1 + v2))) <= 1e-9 * np.max(np.abs(v12))


def test_vcycle_reduces_the_error(blackoil_system):
    """One V-cycle of A e = d from zero is a good approximation: the
    residual of its result is well below |d| (a contraction)."""
    rp, col, blk, r = blackoil_system
    *_, v = O.amg(rp, col, blk, 200, r)
    res = r - _spmv(rp, col, blk, v, 3)
    assert np.linalg.norm(res) < 0.5 * np.linalg.norm(r)


def test_amg_bicgstab_converges_in_fewer_iterations(blackoil_system):
    rp, col, blk, r = blackoil_system
    p_ilu = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    p_amg = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6,
                                linear_solver=capi.LINSOLVER_AMG, amg_coarsen_target=200)
    s0, x0, it0 = O.bcrs_solve(rp, col, blk, r, p_ilu)
    s1, x1, it1 = O.bcrs_solve(rp, col, blk, r, p_amg)
    assert s0 == 0 and s1 == 0
    assert it1 < it0
    for x in (x0, x1):
        res = r - _spmv(rp, col, blk, x, 3)
        assert np.max(np.abs(res)) <= 1e-6 * np.max(np.abs(r)) * 1.0001
    assert np.max(np.abs(x1 - x0)) <= 1e-4 * np.max(np.abs(x0))


def test_newton_with_amg_reaches_the_ilu_state():
    """Newton through the AMG backend converges to the same state as
    through the ILU(0) backend (both linear solves to 1e-8)."""
    prob = problems.blackoil(12, 10, 4)
    states = []
    for ls in (capi.LINSOLVER_ILU0, capi.LINSOLVER_AMG):
        prm = capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-7, linear_solver=ls,
                                  amg_coarsen_target=100)
        o = O.Oracle(prob, prm)
        st, *_ = o.time_integration(3, 86400.0, fixed_dt=True)
        assert st == 0
        states.append(o.solution()[0])
    scale = np.abs(states[0].reshape(-1, 3)).max(axis=0)
    assert np.max(np.abs((states[1] - states[0]).reshape(-1, 3)) / scale) <= 1e-6


def test_lens_amg_2d():
    """The 2D two-phase lens (2x2 blocks, 5-point pattern) through the AMG
    backend: red-black colouring, fewer iterations than ILU(0)."""
    rp, col, blk, r = _system(problems.lens(), 250.0)
    L, sizes, agg, colors, _ = O.amg(rp, col, blk, coarsen_target=100)
    assert L >= 2 and colors.max() == 1
    p_ilu = capi.default_params(linear_tolerance=1e-8)
    p_amg = capi.default_params(linear_tolerance=1e-8, linear_solver=capi.LINSOLVER_AMG, amg_coarsen_target=100)
    s0, x0, it0 = O.bcrs_solve(rp, col, blk, r, p_ilu)
    s1, x1, it1 = O.bcrs_solve(rp, col, blk, r, p_amg)
    assert s0 == 0 and s1 == 0 and it1 <= it0
    assert np.max(np.abs(x1 - x0)) <= 1e-5 * np.max(np.abs(x0))
