"""CPU checks that pin the oracle independently of its own code.

The reference cannot be built here and its tests pin no numbers, so the
oracle is cross-checked against independent restatements:
  * AD Jacobian vs central finite differences of the oracle's residual
  * discrete conservation: interior fluxes cancel in the volume-weighted sum
  * dune-istl block ILU(0) and the reference's BiCGStab loop re-derived in
    numpy (dense blocks, np.linalg.inv), compared factor by factor
  * a two-cell residual and Jacobian derived symbolically (sympy) from the
    reference's formulas (darcyfluxmodule.hh:183-525,
    immisciblelocalresidual.hh:75-155, fvbaselocalresidual.hh:158-626)
"""
import numpy as np
import pytest

import oracle as O
from gbfv import capi, problems


def _lens_state(steps=5, flux="darcy"):
    prob = problems.lens(flux=flux)
    prm = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    st, *_ = orc.time_integration(steps, 250.0)
    assert st == 0
    return prob, prm, orc


@pytest.mark.parametrize("flux", ["darcy", "trans"])
def test_ad_jacobian_matches_central_differences(flux):
    prob, prm, orc = _lens_state(flux=flux)
    x0, m0 = orc.solution()
    dt = 300.0
    orc.linearize(dt, 0)              # fixes the storage cache at x0
    orc.linearize(dt, 1)
    rp, col, J = orc.jacobian()
    N = prob.num_cells
    sw = x0.reshape(-1, 2)[:, 1]
    cand = np.where((sw > 0.3) & (sw < 0.9))[0]
    assert len(cand) >= 10
    rng = np.random.default_rng(0)
    checked = 0
    for I in rng.choice(cand, 10, replace=False):
        for pv, h in ((0, 1e-2), (1, 1e-7)):
            xp = x0.copy(); xp[2 * I + pv] += h
            xm = x0.copy(); xm[2 * I + pv] -= h
            orc.set_solution(xp); orc.linearize(dt, 1); rp_ = orc.residual()
            orc.set_solution(xm); orc.linearize(dt, 1); rm_ = orc.residual()
            fd = (rp_ - rm_) / (2 * h)
            ad = np.zeros(2 * N)
            for r in range(N):
                for k in range(rp[r], rp[r + 1]):
                    if col[k] == I:
                        ad[2 * r:2 * r + 2] = J[k][:, pv]
            scale = np.max(np.abs(ad))
            assert np.max(np.abs(fd - ad)) <= 2e-5 * scale, (I, pv)
            checked += 1
    orc.set_solution(x0, m0)
    assert checked == 20


@pytest.mark.parametrize("which", ["lens", "lens-trans", "blackoil"])
def test_interior_fluxes_cancel(which):
    if which.startswith("lens"):
        flux = "trans" if which == "lens-trans" else "darcy"
        prob = problems.lens(flux=flux)
        prob.bface_type[:] = capi.BC_NOFLOW
        _, _, o = _lens_state(3, flux)
        state = o.solution()
    else:
        prob = problems.blackoil(8, 7, 3)
        prob.constraint[:] = -1
        state = (prob.init_pv.copy(), prob.init_meaning.copy())
        state[0].reshape(-1, 3)[:, 1] += np.linspace(0, 2e6, prob.num_cells)
    prm = capi.default_params()
    orc = O.Oracle(prob, prm)
    orc.set_solution(*state)
    orc.linearize(1000.0, 0)          # storage term vanishes at iteration 0
    r = orc.residual().reshape(-1, prob.b)
    sc = orc.residual_scale().reshape(-1, prob.b)
    V = prob.volume[:, None]
    tot = np.abs((r * V).sum(0))
    assert np.all(tot <= 1e-11 * (sc * V).sum(0)), tot


def _np_ilu0(rp, col, blk):
    """Block ILU(0), natural order, inverse pivots (dune-istl algorithm)."""
    F = blk.copy()
    n = len(rp) - 1
    diag = [next(k for k in range(rp[i], rp[i + 1]) if col[k] == i) for i in range(n)]
    for i in range(n):
        for ij in range(rp[i], rp[i + 1]):
            j = col[ij]
            if j >= i:
                break
            jj = diag[j]
            F[ij] = F[ij] @ F[jj]
            for ik in range(ij + 1, rp[i + 1]):
                for jk in range(jj + 1, rp[j + 1]):
                    if col[ik] == col[jk]:
                        F[ik] = F[ik] - F[ij] @ F[jk]
        F[diag[i]] = np.linalg.inv(F[diag[i]])
    return F, diag


def _np_ilu_apply(rp, col, F, diag, d, b):
    n = len(rp) - 1
    v = np.zeros((n, b))
    dd = d.reshape(n, b)
    for i in range(n):
        rhs = dd[i].copy()
        for k in range(rp[i], diag[i]):
            rhs -= F[k] @ v[col[k]]
        v[i] = rhs
    for i in range(n - 1, -1, -1):
        rhs = v[i].copy()
        for k in range(rp[i + 1] - 1, diag[i], -1):
            rhs -= F[k] @ v[col[k]]
        v[i] = F[diag[i]] @ rhs
    return v.ravel()


def _np_bicgstab(rp, col, A, F, diag, b, bs, tol, abstol, maxit):
    """bicgstabsolver.hh:120-330 with CombinedCriterion (max-norm)."""
    n = len(rp) - 1

    def mv(x):
        y = np.zeros((n, bs))
        xx = x.reshape(n, bs)
        for i in range(n):
            for k in range(rp[i], rp[i + 1]):
                y[i] += A[k] @ xx[col[k]]
        return y.ravel()

    x = np.zeros_like(b)
    r = b.copy()
    init = max(np.max(np.abs(r)), np.finfo(float).tiny * 1e10)
    conv = lambda e: e / max(1e-20, init) <= tol or e <= abstol  # noqa: E731
    if conv(init):
        return x, 0
    r0 = b.copy()
    rho = alpha = omega = 1.0
    v = np.zeros_like(b)
    p = np.zeros_like(b)
    for it in range(maxit):
        rho_i = r0 @ r
        beta = (rho_i / rho) * (alpha / omega)
        rho = rho_i
        p = r + (-beta) * (omega * v - p)
        y = _np_ilu_apply(rp, col, F, diag, p, bs)
        v = mv(y)
        alpha = rho_i / (r0 @ v)
        x = x + alpha * y
        r = r - alpha * v
        if conv(np.max(np.abs(r))):
            return x, it
        z = _np_ilu_apply(rp, col, F, diag, r, bs)
        t = mv(z)
        omega = (t @ r) / (t @ t)
        x = x + omega * z
        r = r - omega * t
    return x, maxit


def _small_system():
    prob = problems.blackoil(5, 4, 3)
    prm = capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    orc.linearize(86400.0, 0)
    rp, col, J = orc.jacobian()
    return prm, rp, col, J, orc.residual()


def test_ilu0_factors_match_numpy_restatement():
    prm, rp, col, J, r = _small_system()
    st, F, v = O.ilu0(rp, col, J, r)
    assert st == 0
    Fn, diag = _np_ilu0(rp, col, J)
    scale = np.maximum(np.abs(Fn).max(axis=(1, 2)), 1e-300)[:, None, None]
    assert np.max(np.abs(F - Fn) / scale) < 1e-11
    vn = _np_ilu_apply(rp, col, Fn, diag, r, 3)
    assert np.max(np.abs(v - vn)) <= 1e-11 * np.max(np.abs(vn))


def test_bicgstab_matches_numpy_restatement():
    prm, rp, col, J, r = _small_system()
    st, x, it = O.bcrs_solve(rp, col, J, r, prm)
    assert st == 0
    Fn, diag = _np_ilu0(rp, col, J)
    xn, itn = _np_bicgstab(rp, col, J, Fn, diag, r, 3, prm.linear_tolerance, 1e-8, 1000)
    assert it == itn
    assert np.max(np.abs(x - xn)) <= 1e-9 * np.max(np.abs(xn))


def test_two_cell_residual_matches_symbolic_derivation():
    sp = pytest.importorskip("sympy")
    # 1x2 vertical lens grid: cell 0 at y=1 (background), cell 1 at y=3 (lens)
    prob = problems.lens(nx=1, ny=2)
    prob.bface_type[:] = capi.BC_NOFLOW
    prm = capi.default_params()
    orc = O.Oracle(prob, prm)
    x = np.array([1.3e5, 0.62, 1.1e5, 0.71])
    orc.set_solution(x)
    dt = 500.0
    orc.linearize(dt, 0)
    orc.linearize(dt, 1)  # storage cache = storage(x) -> only fluxes + zero storage change
    r0 = orc.residual()
    rp, col, J = orc.jacobian()
    # symbolic restatement
    R = sp.Rational
    pw0, S0 = sp.symbols("pw0 S0")
    mats = {0: (R(5, 100), R(37, 10000), R(47, 10)), 1: (R(18, 100), R(45, 100000), R(73, 10))}

    def vg(S, m_id):
        swr, alpha, n = mats[m_id]
        m = 1 - 1 / n
        Se = (S - swr) / (1 - swr)
        pc = ((Se ** (-1 / m) - 1) ** (1 / n)) / alpha
        krw = sp.sqrt(Se) * (1 - (1 - Se ** (1 / m)) ** m) ** 2
        krn = (1 - Se) ** R(1, 3) * (1 - Se ** (1 / m)) ** (2 * m)
        return pc, krw, krn

    rho = (R(1000), R(1460))
    mu = (R(1, 1000), R(57, 100000))
    g = R(-981, 100)
    K = 2 * R(905, 10 ** 14) * R(46, 10 ** 11) / (R(905, 10 ** 14) + R(46, 10 ** 11))
    area, V, phi = R(6), R(12), R(4, 10)
    pw1, S1 = R(11, 1) * 10 ** 4, R(71, 100)
    pc0, krw0, krn0 = vg(S0, 0)
    pc1, krw1, krn1 = vg(S1, 1)
    p_I = (pw0, pw0 + pc0)
    p_J = (pw1, pw1 + pc1)
    lam_I = (krw0 / mu[0], krn0 / mu[1])
    lam_J = (krw1 / mu[0], krn1 / mu[1])
    subs = {pw0: sp.Rational(13, 1) * 10 ** 4, S0: R(62, 100)}
    res0 = []
    dres1 = []
    for a in range(2):
        # gradient along +y between centres y=1 and y=3 (distance 2), face at y=2
        pStatIn = -rho[a] * (g * (1 - 2))
        pStatEx = -rho[a] * (g * (3 - 2))
        pg = (p_J[a] - p_I[a]) * R(2, 4) + 2 * ((pStatEx - pStatIn) / 4)
        up_interior = not (float(pg.subs(subs)) > 0)
        mob = lam_I[a] if up_interior else lam_J[a].subs({})
        flux = (-mob * K * pg) * rho[a] * area
        res0.append(flux / V)
        dres1.append(-flux / V)
    ref_r = [float(e.subs(subs)) for e in res0]
    assert np.allclose(r0[:2], ref_r, rtol=1e-12, atol=0)
    # Jacobian blocks (0,0) = d res0 / d x0 and (1,0) = d res1 / d x0
    blk = {(i, col[k]): J[k] for i in range(2) for k in range(rp[i], rp[i + 1])}
    for a in range(2):
        for v, s in enumerate((pw0, S0)):
            d00 = float(sp.diff(res0[a], s).subs(subs))
            d10 = float(sp.diff(dres1[a], s).subs(subs))
            # storage derivative: phi * rho * dS/dx * V/dt / V
            if v == 1:
                d00 += float((phi * rho[a] * (1 if a == 0 else -1)) / dt)
            assert np.isclose(blk[(0, 0)][a, v], d00, rtol=1e-11, atol=0), (a, v)
            assert np.isclose(blk[(1, 0)][a, v], d10, rtol=1e-11, atol=0), (a, v)


def test_two_cell_trans_residual_matches_symbolic_derivation():
    """transfluxmodule.hh:201-318, 425-456 on a 1x2 vertical lens column."""
    sp = pytest.importorskip("sympy")
    prob = problems.lens(nx=1, ny=2, flux="trans")
    prob.bface_type[:] = capi.BC_NOFLOW
    prm = capi.default_params()
    orc = O.Oracle(prob, prm)
    x = np.array([1.3e5, 0.62, 1.1e5, 0.71])
    orc.set_solution(x)
    dt = 500.0
    orc.linearize(dt, 0)
    orc.linearize(dt, 1)
    r0 = orc.residual()
    R = sp.Rational
    pw0, S0 = sp.symbols("pw0 S0")
    mats = {0: (R(5, 100), R(37, 10000), R(47, 10)), 1: (R(18, 100), R(45, 100000), R(73, 10))}

    def vg(S, m_id):
        swr, alpha, n = mats[m_id]
        m = 1 - 1 / n
        Se = (S - swr) / (1 - swr)
        pc = ((Se ** (-1 / m) - 1) ** (1 / n)) / alpha
        krw = sp.sqrt(Se) * (1 - (1 - Se ** (1 / m)) ** m) ** 2
        krn = (1 - Se) ** R(1, 3) * (1 - Se ** (1 / m)) ** (2 * m)
        return pc, krw, krn

    rho = (R(1000), R(1460))
    mu = (R(1, 1000), R(57, 100000))
    g = R(-981, 100)
    K0, K1 = R(46, 10 ** 11), R(905, 10 ** 14)     # background below, lens above
    half = 1                                          # half cell height (cells 2 m high)
    T0, T1 = K0 * half / half ** 2, K1 * half / half ** 2
    T = T0 * T1 / (T0 + T1)
    area, V = R(6), R(12)
    pw1, S1 = R(11, 1) * 10 ** 4, R(71, 100)
    pc0, krw0, krn0 = vg(S0, 0)
    pc1, krw1, krn1 = vg(S1, 1)
    p_I = (pw0, pw0 + pc0)
    p_J = (pw1, pw1 + pc1)
    lam_I = (krw0 / mu[0], krn0 / mu[1])
    lam_J = (krw1 / mu[0], krn1 / mu[1])
    subs = {pw0: R(13, 1) * 10 ** 4, S0: R(62, 100)}
    distZ = 1 - 3
    ref = []
    for a in range(2):
        rhoAvg = (rho[a] + rho[a]) / 2
        pd = p_J[a] + rhoAvg * (distZ * g) - p_I[a]
        up_interior = not (float(pd.subs(subs)) > 0)
        mob = lam_I[a] if up_interior else lam_J[a]
        flux = pd * mob * (-T) * rho[a] * area
        ref.append(float((flux / V).subs(subs)))
    assert np.allclose(r0[:2], ref, rtol=1e-12, atol=0)
