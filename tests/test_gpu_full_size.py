"""Parity at the benchmark's full sizes against the oracle's logs of the same
runs (tests/golden/*_log.npz, made by tests/golden/make_full_size_golden.py).

100x100x20 black-oil (200k cells, 10 one-day steps, BiCGStab + ILU(0) to
1e-6, Newton tolerance 1e-6): the FP64 and the mixed-precision runs have the
oracle's Newton counts per step and its meanings at the sampled cells, and
their states agree with the oracle's to the summation-order envelope: the
oracle against itself with nothing changed but the order in which the
BiCGStab scalar products are summed ends ENVELOPE apart
(blackoil_100x100x20_dotorder_log.npz; test_cpu_envelope.py pins that
number), and a correct solver that sums in yet another order (the GPU's
block reductions) may end as far from the oracle; the bar is twice that.
The FP64 total of linear iterations is within LINEAR_TOTAL_RTOL of the
oracle's, twice what the summation order alone moves it.  The GPU's final
state is also converged by the oracle's own residual.
Tighter solves shrink the gap: linear 1e-10 / Newton 1e-8 (two steps) to
STATE_RTOL_TIGHT, linear 1e-12 / Newton 1e-10 to STATE_RTOL_TIGHT12 -- the
1e-8 state bar.
100x100x100 (1M cells, two steps), the largest member of the 256-member
ensemble (two steps of 250 s, solved inside a batch) and the 100x100x20
workload through the AMG backend (two steps, against the oracle's AMG
restatement) are held to the same rules."""
import os

import numpy as np
import pytest

import oracle as O

from gbfv import Batch, Context, capi, problems
from parity import rel_state_diff

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STATE_RTOL_TIGHT = 1e-6
STATE_RTOL_TIGHT12 = 1e-8
LINEAR_TOTAL_RTOL = 0.03


def _gold(name):
    return np.load(os.path.join(GOLD, name))


def _envelope():
    """State gap of two oracle runs of the 100x100x20 workload that differ
    only in the summation order of the scalar products."""
    a, b = _gold("blackoil_100x100x20_newton_log.npz"), _gold("blackoil_100x100x20_dotorder_log.npz")
    return rel_state_diff(a["pv"].ravel(), b["pv"].ravel(), a["pv"].shape[1])


def _bench_params(precision):
    return capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=precision,
                               inner_tolerance=1e-6)


def _check_against(g, nits, dts, x, m, bar):
    assert np.array_equal(nits, g["newton"]), (nits, g["newton"])
    assert np.array_equal(dts, g["dt"][:len(dts)])
    idx = g["cells"]
    b = g["pv"].shape[1]
    if b == 3:
        assert np.array_equal(m[idx], g["meaning"])
    diff = rel_state_diff(x.reshape(-1, b)[idx].ravel(), g["pv"].ravel(), b)
    assert diff <= bar, (diff, bar)
    return diff


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_blackoil_100x100x20_against_the_oracle_log(built, precision):
    g = _gold("blackoil_100x100x20_newton_log.npz")
    prob = problems.blackoil(100, 100, 20)
    prm = _bench_params(precision)
    ctx = Context(prob, prm)
    st, dts, nits, lits, _ = ctx.time_integration(9, 86400.0, fixed_dt=True)
    assert st == 0
    x9, m9 = ctx.solution()
    st, rep = ctx.newton_apply(86400.0)
    assert st == 0
    nits = np.append(nits, rep.iterations)
    lits = np.append(lits, rep.linear_iterations)
    x, m = ctx.solution()
    ctx.close()
    _check_against(g, nits, dts, x, m, 2 * _envelope())
    # the oracle's residual at the GPU's last step (old level: the GPU's step-9 state)
    orc = O.Oracle(prob, prm)
    orc.set_solution(x9, m9)
    assert orc.linearize(86400.0, 0) == 0
    orc.set_solution(x, m)
    assert orc.linearize(86400.0, 1) == 0
    err = orc.newton_error()
    assert err <= prm.newton_tolerance, err
    if precision == capi.PREC_FP64:
        assert abs(int(lits.sum()) - int(g["linear"].sum())) <= LINEAR_TOTAL_RTOL * g["linear"].sum(), \
            (lits, g["linear"])


@pytest.mark.parametrize("name,lin,newton,bar", [
    ("blackoil_100x100x20_tight_log.npz", 1e-10, 1e-8, STATE_RTOL_TIGHT),
    ("blackoil_100x100x20_tight12_log.npz", 1e-12, 1e-10, STATE_RTOL_TIGHT12),
])
def test_blackoil_100x100x20_tight_solves_match_the_oracle_state(built, name, lin, newton, bar):
    g = _gold(name)
    prob = problems.blackoil(100, 100, 20)
    prm = capi.default_params(linear_tolerance=lin, newton_tolerance=newton)
    ctx = Context(prob, prm)
    st, dts, nits, lits, _ = ctx.time_integration(len(g["newton"]), 86400.0, fixed_dt=True)
    x, m = ctx.solution()
    ctx.close()
    assert st == 0
    _check_against(g, nits, dts, x, m, bar)


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_blackoil_100x100x100_against_the_oracle_log(built, precision):
    g = _gold("blackoil_100x100x100_newton_log.npz")
    prob = problems.blackoil(100, 100, 100)
    ctx = Context(prob, _bench_params(precision))
    st, dts, nits, lits, _ = ctx.time_integration(len(g["newton"]), 86400.0, fixed_dt=True)
    x, m = ctx.solution()
    ctx.close()
    assert st == 0
    _check_against(g, nits, dts, x, m, 2 * _envelope())
    if precision == capi.PREC_FP64:
        assert abs(int(lits.sum()) - int(g["linear"].sum())) <= LINEAR_TOTAL_RTOL * g["linear"].sum() + 10, \
            (lits, g["linear"])


@pytest.mark.parametrize("precision", [capi.PREC_FP64, capi.PREC_MIXED])
def test_blackoil_100x100x20_amg_against_the_oracle_log(built, precision):
    """The benchmark workload's first two steps through the AMG backend
    (the oracle's restatement, blackoil_100x100x20_amg_log.npz): the same
    Newton counts and meanings, the state within the summation-order
    envelope, the FP64 linear iterations within a few of the oracle's."""
    g = _gold("blackoil_100x100x20_amg_log.npz")
    prob = problems.blackoil(100, 100, 20)
    prm = _bench_params(precision)
    prm.linear_solver = capi.LINSOLVER_AMG
    ctx = Context(prob, prm)
    st, dts, nits, lits, _ = ctx.time_integration(len(g["newton"]), 86400.0, fixed_dt=True)
    x, m = ctx.solution()
    ctx.close()
    assert st == 0
    _check_against(g, nits, dts, x, m, 2 * _envelope())
    if precision == capi.PREC_FP64:
        assert abs(int(lits.sum()) - int(g["linear"].sum())) <= 0.05 * g["linear"].sum() + 2, (lits, g["linear"])


def test_largest_ensemble_member_in_a_batch_against_the_oracle_log(built):
    """The largest realization of the benchmark's ensemble, solved inside a
    batch beside two small members (mixed precision, as the ensemble runs),
    against the oracle's FP64 log of it alone."""
    import sys
    sys.path.insert(0, GOLD)
    from make_full_size_golden import largest_ensemble_member
    g = _gold("ensemble_member_largest_log.npz")
    big, _ = largest_ensemble_member()
    small = [problems.ensemble_member(n, 7 + i, 1.0) for i, n in enumerate((4000, 9000))]
    prm = _bench_params(capi.PREC_MIXED)
    B = Batch([small[0], big, small[1]], prm, cluster_size=4)
    assert B.time_integration(len(g["newton"]), 250.0, fixed_dt=True) == 0
    st, sdt, sn, sl, _ = B.report(1)
    x, m = B.systems[1].solution()
    B.close()
    assert st == 0
    _check_against(g, sn, sdt, x, m, 2 * _envelope())
