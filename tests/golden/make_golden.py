"""Generate the golden fixtures in this directory with the oracle.

The reference publishes no numeric fixtures (its tests only check that an
output file exists), so these are the oracle's answers on small inputs,
frozen so that any later change of the oracle or the kernels shows up:
    lens_6x4.npz      lens problem 6x4, linearization at the initial state
                      and after 3 time steps; 8-step Newton/dt history
    blackoil_5x4x3.npz black-oil 5x4x3 with wells: linearization at the
                      initial state and after 2 one-day steps; Newton counts
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "opm-models_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from gbfv import capi, problems  # noqa: E402


def lin(orc, dt, it):
    assert orc.linearize(dt, it) == 0
    rp, col, J = orc.jacobian()
    return orc.residual(), orc.residual_scale(), rp, col, J


def lens():
    prob = problems.lens(nx=6, ny=4)
    prm = capi.default_params(linear_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    r0, s0, rp, col, J0 = lin(orc, 250.0, 0)
    st, dts, nits, lits, _ = orc.time_integration(3, 250.0)
    assert st == 0
    x3, m3 = orc.solution()
    orc.set_solution(x3)
    lin(orc, 300.0, 0)  # storage cache = storage(x3)
    r3, s3, _, _, J3 = lin(orc, 300.0, 1)
    orc2 = O.Oracle(prob, prm)
    st, dts8, n8, l8, _ = orc2.time_integration(8, 250.0)
    assert st == 0
    x8, _ = orc2.solution()
    np.savez(os.path.join(HERE, "lens_6x4.npz"), r0=r0, s0=s0, rp=rp, col=col, J0=J0,
             x3=x3, r3=r3, s3=s3, J3=J3, dts8=dts8, n8=n8, x8=x8)


def blackoil():
    prob = problems.blackoil(5, 4, 3)
    prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6)
    orc = O.Oracle(prob, prm)
    r0, s0, rp, col, J0 = lin(orc, 86400.0, 0)
    st, dts, n2, l2, _ = orc.time_integration(2, 86400.0, fixed_dt=True)
    assert st == 0
    x2, m2 = orc.solution()
    orc.set_solution(x2, m2)
    lin(orc, 86400.0, 0)  # storage cache = storage(x2)
    r2, s2, _, _, J2 = lin(orc, 86400.0, 1)
    np.savez(os.path.join(HERE, "blackoil_5x4x3.npz"), r0=r0, s0=s0, rp=rp, col=col, J0=J0,
             x2=x2, m2=m2, r2=r2, s2=s2, J2=J2, n2=n2)


if __name__ == "__main__":
    lens()
    blackoil()
    print("golden fixtures written")
