"""Generate the restart-file fixtures in this directory with the oracle.

The reference ships no restart files, so these are the text of the
reference's restart layout (oracle/restart_text.py, a restatement of
opm/models/io/restart.hh and the serialize functions it calls) for states
the oracle computes, frozen so that any later change of the formatter shows
up:
    restart_lens_6x4.ers        lens 6x4 after 3 time steps of 250 s
    restart_blackoil_5x4x3.ers  black-oil 5x4x3 after 2 one-day steps
Run from the repository root:  python tests/golden/make_restart_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "opm-models_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
import restart_text as R  # noqa: E402
from gbfv import capi, problems  # noqa: E402
from gbfv.restart import cartesian_counts  # noqa: E402


def states():
    """(name, pv [N, b], gas meanings or None, grid shape, time, step index)"""
    prob = problems.lens(nx=6, ny=4)
    orc = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6))
    st, dts, _, _, _ = orc.time_integration(3, 250.0)
    assert st == 0
    x, _ = orc.solution()
    yield "restart_lens_6x4.ers", x.reshape(-1, 2), None, (6, 4), float(np.sum(dts)), 3
    prob = problems.blackoil(5, 4, 3)
    orc = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6))
    st, dts, _, _, _ = orc.time_integration(2, 86400.0, fixed_dt=True)
    assert st == 0
    x, m = orc.solution()
    yield "restart_blackoil_5x4x3.ers", x.reshape(-1, 3), m, (5, 4, 3), 2 * 86400.0, 2


def main():
    for name, pv, gm, shape, t, k in states():
        edges, verts = cartesian_counts(shape)
        txt = R.format_restart(pv, gm, num_edges=edges, num_vertices=verts, time=t, time_step_index=k)
        with open(os.path.join(HERE, name), "wb") as f:
            f.write(txt)
        print(name, len(txt), "bytes")


if __name__ == "__main__":
    main()
