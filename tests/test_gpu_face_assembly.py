"""The face-parallel element linearization (a lane per intersection, the
cell's state staged in shared memory, the faces summed in intersection
order from warp shuffles) against the cell-parallel one
(GBFV_CELL_ASSEMBLY=1): residual and Jacobian equal to the bit, for the
2D lens (Darcy and transmissibility flux modules), a 3D two-phase grid and
the black-oil model (element and TPFA linearizers), at Newton iterations 0
and 1 of a state with flow."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, "opm-models_gb300")
from gbfv import Context, capi, problems
cases = {
    "lens": (problems.lens(), capi.default_params(), 250.0),
    "lens_trans": (problems.lens(flux="trans"), capi.default_params(), 250.0),
    "lens3d": (problems.lens(dim=3, nx=12, ny=8, nz=6), capi.default_params(), 250.0),
    "member3d": (problems.ensemble_member(3000, 7, 1.0), capi.default_params(), 250.0),
    "blackoil": (problems.blackoil(9, 7, 4), capi.default_params(), 86400.0),
    "tpfa": (problems.blackoil(9, 7, 4, with_wells=False),
             capi.default_params(linearizer=capi.LINEARIZER_TPFA), 86400.0),
}
out = {}
for name, (prob, prm, dt) in cases.items():
    ctx = Context(prob, prm)
    st = ctx.time_integration(2, dt, fixed_dt=True)[0]
    assert st == 0, (name, st)
    for it in (0, 1):
        assert ctx.linearize(dt, it) == 0
        out["%s_%d_r" % (name, it)] = ctx.residual()
        out["%s_%d_j" % (name, it)] = ctx.jacobian()[2]
    ctx.close()
np.savez(sys.argv[1], **out)
"""


def _run(tmp_path, cell):
    path = str(tmp_path / ("cell.npz" if cell else "face.npz"))
    env = dict(os.environ)
    env.pop("GBFV_CELL_ASSEMBLY", None)
    if cell:
        env["GBFV_CELL_ASSEMBLY"] = "1"
    r = subprocess.run([sys.executable, "-c", SCRIPT, path], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


def test_face_parallel_assembly_equals_the_cell_parallel_one(built, tmp_path):
    face = _run(tmp_path, False)
    cell = _run(tmp_path, True)
    assert sorted(face.files) == sorted(cell.files)
    for k in face.files:
        assert np.array_equal(face[k], cell[k]), k
