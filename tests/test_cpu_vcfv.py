"""CPU checks of the vertex-centred (VCFV) restatement in the oracle
(oracle/vcfv.hh: VcfvStencil, P1 / two-point gradients, the element loop
with one AD focus per corner): the sub-control volumes tile the domain,
its Jacobian is the derivative of its residual, the fluxes cancel between
the two sides of every sub-control-volume face, a hydrostatic column is at
rest, and Newton converges through it on the lens problem.  The GPU form
is compared with these in tests/test_gpu_vcfv.py."""
import numpy as np
import pytest

import oracle as O
from gbfv import capi, problems


def _prm(**kw):
    return capi.default_params(linear_tolerance=1e-8, **kw)


def _perturbed(prob, seed=2):
    rng = np.random.default_rng(seed)
    pv = prob.init_pv.reshape(-1, 2).copy()
    pv[:, 1] = rng.uniform(0.6, 1.0, len(pv))
    pv[:, 0] *= 1.0 + 1e-3 * rng.standard_normal(len(pv))
    return pv.ravel()


def _column(rp, col, blk, i, v):
    n = len(rp) - 1
    out = np.zeros(2 * n)
    for row in range(n):
        for k in range(rp[row], rp[row + 1]):
            if col[k] == i:
                out[2 * row:2 * row + 2] = blk[k][:, v]
    return out


def test_sub_control_volumes_tile_the_domain():
    prob = problems.lens_vcfv(12, 8)
    hx, hy = 6.0 / 12, 4.0 / 8
    o = O.Oracle(prob, _prm())
    assert o.linearize(250.0, 0) == 0
    V = prob.volume.reshape(9, 13)
    assert np.isclose(V.sum(), 24.0, rtol=1e-14)
    assert np.allclose(V[1:-1, 1:-1], hx * hy, rtol=1e-14)
    assert np.allclose(V[0, 1:-1], hx * hy / 2, rtol=1e-14)
    assert np.isclose(V[0, 0], hx * hy / 4, rtol=1e-14)


def test_pattern_is_the_nine_point_vertex_neighbourhood():
    nx, ny = 6, 4
    o = O.Oracle(problems.lens_vcfv(nx, ny), _prm())
    rp, col, _ = o.jacobian()
    mx = nx + 1
    for v in range(len(rp) - 1):
        x, y = v % mx, v // mx
        want = sorted(xx + mx * yy for yy in range(y - 1, y + 2) for xx in range(x - 1, x + 2)
                      if 0 <= xx <= nx and 0 <= yy <= ny)
        assert list(col[rp[v]:rp[v + 1]]) == want


@pytest.mark.parametrize("p1", [True, False])
def test_jacobian_is_the_derivative_of_the_residual(p1):
    prob = problems.lens_vcfv(12, 8, p1=p1)
    o = O.Oracle(prob, _prm())
    assert o.linearize(250.0, 0) == 0
    pv = _perturbed(prob)
    o.set_solution(pv, prob.init_meaning)
    assert o.linearize(250.0, 1) == 0
    r0 = o.residual()
    rp, col, blk = o.jacobian()
    for i in (0, 7, 40, 58, 116):
        for v in range(2):
            h = 1e-7 * max(1.0, abs(pv[2 * i + v]))
            pv2 = pv.copy()
            pv2[2 * i + v] += h
            o.set_solution(pv2, prob.init_meaning)
            assert o.linearize(250.0, 1) == 0
            fd = (o.residual() - r0) / h
            J = _column(rp, col, blk, i, v)
            assert np.max(np.abs(fd - J)) <= 1e-5 * np.max(np.abs(J)), (i, v)


def _no_flow(prob):
    prob.bface_type = np.zeros_like(prob.bface_type)
    return prob


def test_fluxes_cancel_across_faces():
    """With no-flow boundaries and the storage term zero (iteration 0), the
    volume-weighted residuals sum to zero: every sub-control-volume face's
    flux enters its two vertices with opposite signs."""
    prob = _no_flow(problems.lens_vcfv(12, 8))
    o = O.Oracle(prob, _prm())
    o.set_solution(_perturbed(prob), prob.init_meaning)
    assert o.linearize(250.0, 0) == 0
    r = o.residual().reshape(-1, 2) * prob.volume[:, None]
    sc = o.residual_scale().reshape(-1, 2) * prob.volume[:, None]
    assert np.all(np.abs(r.sum(axis=0)) <= 1e-12 * sc.sum(axis=0))


@pytest.mark.parametrize("p1", [True, False])
def test_hydrostatic_column_is_at_rest(p1):
    """The initial hydrostatic water column with closed boundaries: the P1
    (and two-point) pressure gradient balances the gravity correction on
    every face, so the residual vanishes to rounding."""
    prob = _no_flow(problems.lens_vcfv(12, 8, p1=p1))
    o = O.Oracle(prob, _prm())
    assert o.linearize(250.0, 0) == 0
    r = o.residual()
    sc = o.residual_scale()
    assert np.max(np.abs(r)) <= 1e-10 * np.max(sc)


def test_newton_converges_through_vcfv():
    prob = problems.lens_vcfv()
    o = O.Oracle(prob, _prm())
    st, dt, nn, nl, _ = o.time_integration(6, 250.0)
    assert st == 0 and np.all(nn >= 1) and np.all(nn <= 12)
    pv, _ = o.solution()
    sw = pv.reshape(-1, 2)[:, 1]
    assert np.all(np.isfinite(pv)) and sw.min() < 0.999 and sw.max() <= 1.0 + 1e-12


def test_amg_backend_solves_the_vcfv_pattern():
    """The system of the lens after three time steps (infiltrating NAPL):
    BiCGStab with AMG reaches the ILU(0) solution."""
    prob = problems.lens_vcfv()
    prm = _prm()
    o = O.Oracle(prob, prm)
    assert o.time_integration(3, 250.0)[0] == 0
    assert o.linearize(250.0, 0) == 0
    rp, col, blk = o.jacobian()
    r = o.residual()
    s1, x1, it1 = O.bcrs_solve(rp, col, blk, r, prm)
    prm2 = _prm(linear_solver=capi.LINSOLVER_AMG, amg_coarsen_target=100)
    s2, x2, it2 = O.bcrs_solve(rp, col, blk, r, prm2)
    assert s1 == 0 and s2 == 0
    assert np.max(np.abs(x1 - x2)) <= 1e-5 * np.max(np.abs(x1))


@pytest.mark.parametrize("method", [1, 0, -1])
def test_fd_jacobian_approximates_the_ad_one(method):
    """The finite-difference local linearizer on the vertex-centred stencil
    (lens_immiscible_vcfv_fd): the same residual as the AD linearizer, a
    Jacobian within the differencing error of the AD one."""
    prob = problems.lens_vcfv(12, 8)
    pv = _perturbed(prob)
    out = []
    for lin in (capi.LIN_AD, capi.LIN_FD):
        o = O.Oracle(prob, _prm(local_linearizer=lin, numeric_difference_method=method))
        assert o.linearize(250.0, 0) == 0
        o.set_solution(pv, prob.init_meaning)
        assert o.linearize(250.0, 1) == 0
        out.append((o.residual(), o.jacobian()[2]))
    (ra, ja), (rf, jf) = out
    assert np.array_equal(ra, rf)
    scale = np.max(np.abs(ja), axis=0)
    # eps ~ 1e-10: the round-off of the residual over eps dominates
    assert np.max(np.abs(jf - ja) / np.maximum(scale, 1e-300)) <= 2e-4


def _bo_state(prob, seed=3):
    """Pressures, water saturations and both gas meanings perturbed."""
    rng = np.random.default_rng(seed)
    pv = prob.init_pv.reshape(-1, 3).copy()
    pv[:, 1] *= 1.0 + 0.01 * rng.standard_normal(len(pv))
    pv[:, 0] = rng.uniform(0.1, 0.3, len(pv))
    m = prob.init_meaning.copy()
    m[::3] = capi.GAS_SG
    pv[::3, 2] = rng.uniform(0.0, 0.2, len(pv[::3]))
    return pv.ravel(), m


def test_blackoil_jacobian_is_the_derivative_of_the_residual():
    """The black-oil model on the vertex-centred stencil (the reference's
    reservoir_blackoil_vcfv): component fluxes with the upstream 1/B and
    R_s, component storage, wells as constraint vertices."""
    prob = problems.blackoil_vcfv(12, 8)
    o = O.Oracle(prob, capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6))
    assert o.linearize(86400.0, 0) == 0
    pv, m = _bo_state(prob)
    o.set_solution(pv, m)
    assert o.linearize(86400.0, 1) == 0
    r0 = o.residual()
    rp, col, blk = o.jacobian()
    n = len(rp) - 1
    for i in (5, 20, 50, 80, 100):
        for v in range(3):
            h = 1e-7 * max(1.0, abs(pv[3 * i + v]))
            pv2 = pv.copy()
            pv2[3 * i + v] += h
            o.set_solution(pv2, m)
            assert o.linearize(86400.0, 1) == 0
            fd = (o.residual() - r0) / h
            J = np.zeros(3 * n)
            for row in range(n):
                for k in range(rp[row], rp[row + 1]):
                    if col[k] == i:
                        J[3 * row:3 * row + 3] = blk[k][:, v]
            assert np.max(np.abs(fd - J)) <= 1e-5 * np.max(np.abs(J)), (i, v)


def test_blackoil_fluxes_cancel_and_newton_converges():
    prob = problems.blackoil_vcfv(12, 8, with_wells=False)
    o = O.Oracle(prob, capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6))
    pv, m = _bo_state(prob)
    o.set_solution(pv, m)
    assert o.linearize(86400.0, 0) == 0
    r = o.residual().reshape(-1, 3) * prob.volume[:, None]
    sc = o.residual_scale().reshape(-1, 3) * prob.volume[:, None]
    assert np.all(np.abs(r.sum(axis=0)) <= 1e-12 * sc.sum(axis=0))
    wells = problems.blackoil_vcfv(12, 8)
    o2 = O.Oracle(wells, capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6))
    st, _, nn, _, _ = o2.time_integration(4, 86400.0, fixed_dt=True)
    assert st == 0 and np.all(nn >= 1) and np.all(nn <= 12)
