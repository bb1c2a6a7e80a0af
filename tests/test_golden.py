"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py):
the oracle must keep reproducing them (CPU), and the CUDA path must match
them through the C ABI (GPU)."""
import os

import numpy as np
import pytest

import oracle as O
from gbfv import capi, problems
from parity import RTOL_LIN, jacobian_mismatch_fast, residual_mismatch

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cases():
    lens = np.load(os.path.join(HERE, "lens_6x4.npz"))
    bo = np.load(os.path.join(HERE, "blackoil_5x4x3.npz"))
    return [
        ("lens", problems.lens(nx=6, ny=4), capi.default_params(linear_tolerance=1e-6), lens,
         [(None, 250.0, 0, "r0", "s0", "J0"), ("x3", 300.0, 1, "r3", "s3", "J3")]),
        ("blackoil", problems.blackoil(5, 4, 3),
         capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6), bo,
         [(None, 86400.0, 0, "r0", "s0", "J0"), ("x2", 86400.0, 1, "r2", "s2", "J2")]),
    ]


def _check(impl_factory, tol):
    for name, prob, prm, g, states in _cases():
        impl = impl_factory(prob, prm)
        for xs, dt, it, rk, sk, jk in states:
            if xs is not None:
                meaning = g["m2"] if name == "blackoil" else None
                if it > 0:  # storage cache from the state itself (iteration 0 first)
                    impl.set_solution(g[xs], meaning)
                    impl.linearize(dt, 0)
                impl.set_solution(g[xs], meaning)
            assert impl.linearize(dt, it) == 0
            rp, col, J = impl.jacobian()
            assert np.array_equal(rp, g["rp"]) and np.array_equal(col, g["col"])
            assert residual_mismatch(impl.residual(), g[rk], g[sk]) <= tol, (name, rk)
            assert jacobian_mismatch_fast(rp, col, J, g[jk]) <= tol, (name, jk)


def test_oracle_reproduces_golden():
    _check(lambda p, prm: O.Oracle(p, prm), 1e-13)


def test_oracle_newton_history_golden():
    g = np.load(os.path.join(HERE, "lens_6x4.npz"))
    orc = O.Oracle(problems.lens(nx=6, ny=4), capi.default_params(linear_tolerance=1e-6))
    st, dts, n, _, _ = orc.time_integration(8, 250.0)
    assert st == 0 and np.array_equal(n, g["n8"]) and np.allclose(dts, g["dts8"], rtol=1e-13)
    x, _ = orc.solution()
    assert np.allclose(x, g["x8"], rtol=1e-10, atol=1e-12)


@pytest.mark.gpu
def test_gpu_reproduces_golden(built):
    from gbfv import Context
    _check(lambda p, prm: Context(p, prm), RTOL_LIN)


@pytest.mark.gpu
def test_gpu_newton_history_golden(built):
    from gbfv import Context
    g = np.load(os.path.join(HERE, "lens_6x4.npz"))
    ctx = Context(problems.lens(nx=6, ny=4), capi.default_params(linear_tolerance=1e-6))
    st, dts, n, _, _ = ctx.time_integration(8, 250.0)
    assert st == 0 and np.array_equal(n, g["n8"]) and np.allclose(dts, g["dts8"], rtol=1e-12)
    x, _ = ctx.solution()
    assert np.max(np.abs(x - g["x8"]) / np.maximum(np.abs(g["x8"]), 1.0)) <= 1e-8
