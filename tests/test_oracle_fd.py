"""The oracle's finite-difference local linearizer (FvBaseFdLocalLinearizer,
fvbasefdlocallinearizer.hh:222-510) against its definition: a diagonal
block column is the element's own residual at the deflected state minus
the one at the other state, divided by the total deflection, where the
element's residual at a state is the global residual's row of that cell
after only that cell's variables changed (the neighbours keep theirs).  The
residual itself is the AD linearizer's; Newton counts match the AD run."""
import numpy as np
import pytest

import oracle as O
from gbfv import capi, problems

BASE_EPS = max(0.9123e-10, np.finfo(float).eps * 1.23e3)


def _pv_weight(model, pv, ref_p, meaning):
    if model == capi.MODEL_IMMISCIBLE_2P:
        return 10 / ref_p if pv == 0 else 1.0
    if pv == 0:
        return 1.0
    if pv == 1:
        return 1.0 / 300e5
    return {capi.GAS_SG: 1.0, capi.GAS_RS: 1.0 / 250., capi.GAS_RV: 1.0 / 0.025}[int(meaning)]


def _state(kind):
    if kind == "lens":
        prob, dt, kw, steps = problems.lens(nx=12, ny=8), 250.0, {}, 4
    else:
        prob, dt, kw, steps = problems.blackoil(6, 5, 3), 86400.0, dict(newton_tolerance=1e-6), 2
    o = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6, **kw))
    assert o.time_integration(steps, dt, fixed_dt=True)[0] == 0
    return prob, dt, kw, o.solution()


@pytest.mark.parametrize("kind", ["lens", "blackoil"])
@pytest.mark.parametrize("method", [1, 0, -1])
def test_diagonal_columns_are_the_deflected_residual_differences(kind, method):
    prob, dt, kw, (x, m) = _state(kind)
    b = prob.b
    prm_fd = capi.default_params(linear_tolerance=1e-6, local_linearizer=capi.LIN_FD,
                                 numeric_difference_method=method, **kw)
    prm_ad = capi.default_params(linear_tolerance=1e-6, **kw)
    fd = O.Oracle(prob, prm_fd)
    fd.set_solution(x, m)
    assert fd.linearize(dt, 0) == 0 and fd.linearize(dt, 1) == 0
    rp, col, J = fd.jacobian()
    r_fd = fd.residual()
    # the residual rows of deflected states; the cache of old storage is filled at x
    ev = O.Oracle(prob, prm_ad)
    ev.set_solution(x, m)
    assert ev.linearize(dt, 0) == 0
    assert ev.linearize(dt, 1) == 0
    assert np.array_equal(ev.residual(), r_fd)
    ref_p = x[0]
    cells = [0, 5, prob.num_cells // 2, prob.num_cells - 1]
    for c in cells:
        diag = [k for k in range(rp[c], rp[c + 1]) if col[k] == c][0]
        for pv in range(b):
            eps = BASE_EPS / _pv_weight(prob.model, pv, ref_p, m[c])
            xs = x.copy()
            i = c * b + pv
            delta = 0.0
            if method >= 0:
                xs[i] += eps
                delta += eps
                ev.set_solution(xs, m)
                ev.linearize(dt, 1)
                hi = ev.residual()[c * b:(c + 1) * b].copy()
            else:
                hi = r_fd[c * b:(c + 1) * b].copy()
            if method <= 0:
                xs[i] -= delta + eps
                delta += eps
                ev.set_solution(xs, m)
                ev.linearize(dt, 1)
                lo = ev.residual()[c * b:(c + 1) * b].copy()
            else:
                lo = r_fd[c * b:(c + 1) * b]
            want = (hi - lo) / delta
            got = J[diag][:, pv]
            # constraint rows are identity
            if prob.constraint[c] >= 0:
                continue
            assert np.array_equal(got, want), (kind, method, c, pv, got, want)
        ev.set_solution(x, m)


@pytest.mark.parametrize("kind", ["lens", "blackoil"])
def test_fd_newton_counts_equal_ad(kind):
    if kind == "lens":
        prob, dt, kw, steps = problems.lens(), 250.0, {}, 6
    else:
        prob, dt, kw, steps = problems.blackoil(10, 8, 4), 86400.0, dict(newton_tolerance=1e-6), 3
    runs = []
    for lin in (capi.LIN_AD, capi.LIN_FD):
        o = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6, local_linearizer=lin, **kw))
        st, _, n, _, _ = o.time_integration(steps, dt, fixed_dt=True)
        assert st == 0
        runs.append((n, o.solution()[0]))
    assert np.array_equal(runs[0][0], runs[1][0])
