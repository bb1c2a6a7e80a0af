"""GPU parity of the TPFA linearizer (params.linearizer = LINEARIZER_TPFA:
TpfaLinearizer + BlackOilLocalResidualTPFA) against the oracle's
restatement: residual and Jacobian at the 1e-12 bar, Newton through it,
and the problems it refuses."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from gbfv import Context, capi, problems
from parity import RTOL_LIN, jacobian_mismatch_fast, rel_state_diff, residual_mismatch

pytestmark = pytest.mark.gpu


def _prm(**kw):
    return capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6, linearizer=capi.LINEARIZER_TPFA, **kw)


def _compare(ctx, orc, dt, it, state=None):
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


def test_tpfa_linearization_matches_the_oracle(built):
    prob = problems.blackoil(9, 7, 4, with_wells=False)
    orc = O.Oracle(prob, _prm())
    ctx = Context(prob, _prm())
    er, ej = _compare(ctx, orc, 86400.0, 0)
    assert er <= RTOL_LIN and ej <= RTOL_LIN, (er, ej)
    # a state with flow in every direction and both gas meanings
    rng = np.random.default_rng(3)
    pv = prob.init_pv.reshape(-1, 3).copy()
    pv[:, 1] *= 1.0 + 0.02 * rng.standard_normal(len(pv))
    pv[:, 0] = rng.uniform(0.1, 0.3, len(pv))
    m = prob.init_meaning.copy()
    m[::3] = capi.GAS_SG
    pv[::3, 2] = rng.uniform(0.0, 0.2, len(pv[::3]))
    for it in (0, 1, 2):
        er, ej = _compare(ctx, orc, 86400.0, it, (pv.ravel(), m))
        assert er <= RTOL_LIN and ej <= RTOL_LIN, (it, er, ej)


def test_tpfa_rows_scale_with_the_volume(built):
    """The element linearizer's rows are the TPFA rows divided by the
    volume where the two flux modules agree -- here checked on the storage
    part alone: a single cell has no faces."""
    p1 = problems.blackoil(1, 1, 1, with_wells=False)
    rs = []
    for lin in (capi.LINEARIZER_ELEMENT, capi.LINEARIZER_TPFA):
        ctx = Context(p1, capi.default_params(linearizer=lin))
        ctx.linearize(86400.0, 0)
        pv = p1.init_pv.copy()
        pv[1] *= 1.01
        ctx.set_solution(pv, p1.init_meaning)
        ctx.linearize(86400.0, 1)
        rs.append(ctx.residual())
    assert np.allclose(rs[1], rs[0] * p1.volume[0], rtol=1e-13, atol=0)


def test_tpfa_newton_matches_the_oracle(built):
    prob = problems.blackoil(12, 10, 4, with_wells=False)
    orc = O.Oracle(prob, _prm())
    ctx = Context(prob, _prm())
    so, dto, no, lo, _ = orc.time_integration(4, 86400.0, fixed_dt=True)
    sg, dtg, ng, lg, _ = ctx.time_integration(4, 86400.0, fixed_dt=True)
    assert so == 0 and sg == 0
    assert np.array_equal(no, ng), (no, ng)
    pvo, mo = orc.solution()
    pvg, mg = ctx.solution()
    assert np.array_equal(mo, mg)
    assert rel_state_diff(pvg, pvo, 3) <= 1e-8


def test_tpfa_refuses_what_it_does_not_model(built):
    # constraint cells (TpfaLinearizer applies none)
    with pytest.raises(RuntimeError, match="ERR_UNSUPPORTED"):
        Context(problems.blackoil(6, 5, 3, with_wells=True), _prm())
    # the immiscible model (no BlackOilLocalResidualTPFA)
    with pytest.raises(RuntimeError, match="ERR_UNSUPPORTED"):
        Context(problems.lens(), _prm())
    # finite differences
    with pytest.raises(RuntimeError, match="ERR_ARG"):
        Context(problems.blackoil(6, 5, 3, with_wells=False), _prm(local_linearizer=capi.LIN_FD))
    # the linearizer is fixed at creation
    ctx = Context(problems.blackoil(6, 5, 3, with_wells=False), _prm())
    assert ctx.lib.gbfv_set_params(ctx.h, C.byref(capi.default_params())) == capi.ERR_UNSUPPORTED
