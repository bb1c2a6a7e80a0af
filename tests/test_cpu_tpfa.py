"""CPU checks of the TPFA linearizer restatement (TpfaLinearizer +
BlackOilLocalResidualTPFA, tpfalinearizer.hh:711-866,
blackoillocalresidualtpfa.hh:234-505) in the oracle: its Jacobian is the
derivative of its residual, the fluxes cancel between the two sides of
every face, the rows are the element linearizer's structure without the
division by the volume, and Newton converges through it.  The GPU form is
compared with these in tests/test_gpu_tpfa.py."""
import numpy as np
import pytest

import oracle as O
from gbfv import capi, problems


def _prm(**kw):
    return capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6,
                               linearizer=capi.LINEARIZER_TPFA, **kw)


def _perturbed_state(prob, seed=5):
    """The initial state with pressures and the gas variable perturbed, so
    that fluxes flow both ways across faces."""
    rng = np.random.default_rng(seed)
    pv = prob.init_pv.reshape(-1, 3).copy()
    pv[:, 1] *= 1.0 + 0.02 * rng.standard_normal(len(pv))
    pv[:, 0] = rng.uniform(0.1, 0.3, len(pv))
    return pv.ravel(), prob.init_meaning


@pytest.fixture(scope="module")
def prob():
    return problems.blackoil(8, 6, 4, with_wells=False)


def test_jacobian_is_the_derivative_of_the_residual(prob):
    o = O.Oracle(prob, _prm())
    pv, m = _perturbed_state(prob)
    o.set_solution(pv, m)
    assert o.linearize(86400.0, 1) == 0
    r0 = o.residual()
    rp, col, blk = o.jacobian()
    n = len(rp) - 1
    rng = np.random.default_rng(1)
    for _ in range(6):
        i = int(rng.integers(n))
        for v in range(3):
            h = 1e-7 * max(1.0, abs(pv[3 * i + v]))
            pv2 = pv.copy()
            pv2[3 * i + v] += h
            o.set_solution(pv2, m)
            assert o.linearize(86400.0, 1) == 0
            fd = (o.residual() - r0) / h
            # column (., i) of the Jacobian: block (row, i) entries [e][v]
            for row in range(n):
                k = [kk for kk in range(rp[row], rp[row + 1]) if col[kk] == i]
                want = blk[k[0]][:, v] if k else np.zeros(3)
                got = fd[3 * row:3 * row + 3]
                scale = np.abs(blk[rp[row]:rp[row + 1]]).max() * h + 1e-12
                assert np.all(np.abs(got - want) <= 1e-3 * np.abs(want) + 1e-3 * scale / h * 1e-3 + 1e-9), \
                    (row, i, v, got, want)
    o.set_solution(pv, m)


def test_fluxes_cancel_across_faces(prob):
    """Each face's flux enters its two rows with opposite signs (evaluated
    from each side), so the sum of all rows is the sum of the storage terms
    to rounding."""
    o = O.Oracle(prob, _prm())
    pv, m = _perturbed_state(prob)
    o.set_solution(pv, m)
    assert o.linearize(86400.0, 0) == 0   # iteration 0: storage equals its cache
    r = o.residual().reshape(-1, 3)
    scale = o.residual_scale().reshape(-1, 3)
    # at iteration 0 the storage term is zero, the residual is the net flux
    assert np.all(np.abs(r.sum(axis=0)) <= 1e-9 * scale.sum(axis=0))


def test_rows_are_the_element_rows_times_the_volume_where_no_flux():
    """With a single cell (no faces) both linearizers reduce to the storage
    term: the TPFA row is the element linearizer's row times the volume."""
    p1 = problems.blackoil(1, 1, 1, with_wells=False)
    pv, m = _perturbed_state(p1)
    res = []
    for lin in (capi.LINEARIZER_ELEMENT, capi.LINEARIZER_TPFA):
        o = O.Oracle(p1, capi.default_params(linearizer=lin))
        o.set_solution(p1.init_pv, m)
        o.linearize(86400.0, 0)
        o.set_solution(pv, m)
        o.linearize(86400.0, 1)
        res.append(o.residual())
    V = p1.volume[0]
    assert np.allclose(res[1], res[0] * V, rtol=1e-13, atol=0)


def test_newton_converges_through_tpfa(prob):
    o = O.Oracle(prob, _prm())
    st, dt, nn, nl, _ = o.time_integration(3, 86400.0, fixed_dt=True)
    assert st == 0 and np.all(nn >= 1) and np.all(nn <= 10)
    pv, _ = o.solution()
    assert np.all(np.isfinite(pv))
