"""GPU checks of restart files written from and read into a context: a run
stopped after k time steps, written to a restart file and continued in a
fresh context from that file ends with the same bits as the run that was
not stopped, and the file equals the restatement's text of the state."""
import numpy as np
import pytest

import restart_text as R
from gbfv import Context, capi, problems, restart

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["lens", "blackoil"])
def test_stop_write_read_continue_equals_straight_run(built, tmp_path, kind):
    if kind == "lens":
        prob, shape, dt = problems.lens(), (48, 32), 250.0
        prm = capi.default_params(linear_tolerance=1e-6)
    else:
        prob, shape, dt = problems.blackoil(16, 12, 5), (16, 12, 5), 86400.0
        prm = capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6, precision=capi.PREC_MIXED,
                                  inner_tolerance=1e-6)
    edges, verts = restart.cartesian_counts(shape)
    a = Context(prob, prm)
    st, _, na, la, _ = a.time_integration(6, dt, fixed_dt=True)
    assert st == 0
    xa, ma = a.solution()
    a.close()

    b = Context(prob, prm)
    st, _, nb1, lb1, _ = b.time_integration(3, dt, fixed_dt=True)
    assert st == 0
    path = str(tmp_path / restart.restart_file_name(".", "gbfv_" + kind, 3 * dt))
    b.write_restart(path, restart.info(edges, verts, time=3 * dt, time_step_index=3))
    xb, mb = b.solution()
    b.close()
    with open(path, "rb") as f:
        text = f.read()
    gm = mb if kind == "blackoil" else None
    assert text == R.format_restart(xb.reshape(-1, prob.b), gm, num_edges=edges, num_vertices=verts,
                                    time=3 * dt, time_step_index=3)

    c = Context(prob, prm)
    out = c.read_restart(path, restart.info(edges, verts))
    assert out.time == 3 * dt and out.time_step_index == 3
    xc0, mc0 = c.solution()
    assert np.array_equal(xc0, xb) and np.array_equal(mc0, mb)
    st, _, nc2, lc2, _ = c.time_integration(3, dt, fixed_dt=True)
    assert st == 0
    assert np.array_equal(np.concatenate([nb1, nc2]), na), (nb1, nc2, na)
    xc, mc = c.solution()
    c.close()
    assert np.array_equal(xc, xa) and np.array_equal(mc, ma)


def test_read_rejects_another_grid(built, tmp_path):
    prob = problems.blackoil(8, 6, 3)
    ctx = Context(prob, capi.default_params())
    path = str(tmp_path / "x.ers")
    edges, verts = restart.cartesian_counts((8, 6, 3))
    ctx.write_restart(path, restart.info(edges, verts))
    with pytest.raises(Exception):
        ctx.read_restart(path, restart.info(edges, verts + 1))
    ctx.close()


def test_vertex_centred_stop_write_read_continue(built, tmp_path):
    """The vertex-centred lens: the context writes its vertices (codim 2,
    the element count in the cookie) and a fresh context continues from the
    file to the bits of the run that was not stopped."""
    prob, dt = problems.lens_vcfv(), 250.0
    prm = capi.default_params(linear_tolerance=1e-8)
    edges, verts = restart.cartesian_counts((48, 32))
    a = Context(prob, prm)
    assert a.time_integration(4, dt, fixed_dt=True)[0] == 0
    xa, _ = a.solution()
    a.close()
    b = Context(prob, prm)
    assert b.time_integration(2, dt, fixed_dt=True)[0] == 0
    path = str(tmp_path / "vcfv.ers")
    b.write_restart(path, restart.info(edges, verts, time=2 * dt, time_step_index=2))
    xb, _ = b.solution()
    b.close()
    with open(path, "rb") as f:
        text = f.read()
    assert text == R.format_restart(xb.reshape(-1, 2), None, num_edges=edges, num_vertices=verts, time=2 * dt,
                                    time_step_index=2, entity_codim=2, num_elements=48 * 32)
    c = Context(prob, prm)
    out = c.read_restart(path, restart.info(edges, verts))
    assert out.time == 2 * dt
    assert c.time_integration(2, dt, fixed_dt=True)[0] == 0
    xc, _ = c.solution()
    c.close()
    assert np.array_equal(xc, xa)
