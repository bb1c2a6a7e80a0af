"""GPU checks of the batched path (gbfv_batch_*): every system of a batch of
uneven ensemble realizations gives exactly the result it gives alone with
the same solver launch configuration -- the same time steps, Newton and
linear iteration counts, and a bit-identical final state -- and agrees with
the CPU oracle on the Newton counts and the state."""
import numpy as np
import pytest

import oracle as O
from gbfv import Batch, Context, capi, problems
from parity import rel_state_diff

pytestmark = pytest.mark.gpu

CLUSTER = 4


def _members(sizes, seed0=1000):
    rng = np.random.default_rng(seed0)
    sig = rng.uniform(0.5, 1.5, len(sizes))
    return [problems.ensemble_member(n, seed0 + i, float(s)) for i, (n, s) in enumerate(zip(sizes, sig))]


def _alone(prob, prm, steps, dt):
    ctx = Context(prob, prm)
    ctx.set_solver_config(prm.precision, 1, CLUSTER)
    st, sdt, sn, sl, _ = ctx.time_integration(steps, dt)
    x, m = ctx.solution()
    ctx.close()
    return st, sdt, sn, sl, x, m


@pytest.mark.parametrize("precision", [capi.PREC_MIXED, capi.PREC_FP64])
def test_batch_equals_alone(built, precision):
    sizes = [3000, 12000, 800, 20000, 6000]
    probs = _members(sizes)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=precision,
                              inner_tolerance=1e-5)
    steps, dt = 3, 200.0
    B = Batch(probs, prm, cluster_size=CLUSTER)
    assert B.stats()["cluster_size"] == CLUSTER
    assert B.time_integration(steps, dt) == 0
    st_b = B.stats()
    assert st_b["rounds"] > 0 and st_b["solve_launches"] > 0 and st_b["graph_launches"] > 0
    for i, p in enumerate(probs):
        bst, bdt, bsn, bsl, _ = B.report(i)
        xb, mb = B.systems[i].solution()
        st, sdt, sn, sl, x, m = _alone(p, prm, steps, dt)
        assert bst == st == 0
        assert np.array_equal(bdt, sdt[:len(bdt)]) and len(bdt) == steps
        assert np.array_equal(bsn, sn) and np.array_equal(bsl, sl), (i, bsn, sn, bsl, sl)
        assert np.array_equal(xb, x) and np.array_equal(mb, m), i
    B.close()


def test_batch_matches_oracle(built):
    probs = _members([2500, 7000], seed0=77)
    prm = capi.default_params(linear_tolerance=1e-8, newton_tolerance=1e-7)
    B = Batch(probs, prm, cluster_size=CLUSTER)
    assert B.time_integration(3, 200.0) == 0
    for i, p in enumerate(probs):
        _, _, bsn, _, _ = B.report(i)
        orc = O.Oracle(p, prm)
        st, _, on, _, _ = orc.time_integration(3, 200.0)
        assert st == 0
        assert np.array_equal(bsn, on), (i, bsn, on)
        xb, _ = B.systems[i].solution()
        xo, _ = orc.solution()
        assert rel_state_diff(xb, xo, 2) <= 1e-8
    B.close()


def test_batch_blackoil_with_wells(built):
    probs = [problems.blackoil(12, 10, 4), problems.blackoil(9, 8, 3, seed=99)]
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                              inner_tolerance=1e-5)
    B = Batch(probs, prm, cluster_size=2)
    assert B.time_integration(3, 86400.0, fixed_dt=True) == 0
    for i, p in enumerate(probs):
        _, _, bsn, bsl, _ = B.report(i)
        ctx = Context(p, prm)
        ctx.set_solver_config(capi.PREC_MIXED, 1, 2)
        st, _, sn, sl, _ = ctx.time_integration(3, 86400.0, fixed_dt=True)
        assert st == 0 and np.array_equal(bsn, sn) and np.array_equal(bsl, sl)
        assert np.array_equal(B.systems[i].solution()[0], ctx.solution()[0])
    B.close()


@pytest.mark.parametrize("precision", [capi.PREC_MIXED, capi.PREC_FP64])
def test_round_is_one_graph_launch_and_equals_the_host_driven_round(built, monkeypatch, precision):
    """The device-driven round (every phase and the per-system decisions
    between them in one captured graph) launches exactly one graph per
    round and gives the host-driven round's results bit for bit: the same
    rounds, steps, Newton and linear iterations and states."""
    probs = _members([3000, 12000, 800, 6000], seed0=31)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=precision,
                              inner_tolerance=1e-5)
    runs = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("GBFV_BATCH_HOST_ROUND", mode)
        B = Batch(probs, prm, cluster_size=CLUSTER)
        st = B.time_integration(3, 200.0)
        stats = B.stats()
        res = [(B.report(i), B.systems[i].solution()) for i in range(len(probs))]
        B.close()
        runs[mode] = (st, stats, res)
    (sh, hs, hres), (sd, ds, dres) = runs["1"], runs["0"]
    assert sh == sd == 0
    assert ds["rounds"] == hs["rounds"] > 0
    assert ds["graph_launches"] == ds["rounds"]
    assert hs["graph_launches"] > hs["rounds"]
    for (hr, (hx, hm)), (dr, (dx, dm)) in zip(hres, dres):
        for a, b in zip(hr, dr):
            assert np.array_equal(np.asarray(a), np.asarray(b)), (a, b)
        assert np.array_equal(hx, dx) and np.array_equal(hm, dm)
