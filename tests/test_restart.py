"""Restart files (CPU): the library's formatter and parser against the
restatement of the reference's layout (oracle/restart_text.py) and the
frozen fixtures; every double reads back to the same bits; malformed files
are rejected; file names as Restart::restartFileName_ makes them."""
import os

import numpy as np
import pytest

import oracle as O
import restart_text as R
from gbfv import capi, problems, restart

HERE = os.path.dirname(os.path.abspath(__file__))


def _oracle_state(kind):
    if kind == "lens":
        prob = problems.lens(nx=12, ny=8)
        orc = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6))
        assert orc.time_integration(2, 250.0)[0] == 0
        x, _ = orc.solution()
        return x.reshape(-1, 2), None, (12, 8)
    prob = problems.blackoil(6, 5, 3)
    orc = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6, newton_tolerance=1e-6))
    assert orc.time_integration(1, 86400.0, fixed_dt=True)[0] == 0
    x, m = orc.solution()
    return x.reshape(-1, 3), m, (6, 5, 3)


@pytest.mark.parametrize("kind", ["lens", "blackoil"])
@pytest.mark.parametrize("vtk", [True, False])
def test_format_equals_restatement(kind, vtk):
    pv, gm, shape = _oracle_state(kind)
    edges, verts = restart.cartesian_counts(shape)
    kw = dict(time=1234.5, time_step_index=7, episode_index=2, episode_start_time=1000.0,
              episode_length=3.1e7, start_time=0.0, vtk_section=vtk, vtk_writer_num=5)
    got = restart.format_restart(restart.info(edges, verts, **kw), pv, gm)
    want = R.format_restart(pv, gm, num_edges=edges, num_vertices=verts, **kw)
    assert got == want


@pytest.mark.parametrize("name,shape,b,t,k", [("restart_lens_6x4.ers", (6, 4), 2, 1105.9027777777778, 3),
                                              ("restart_blackoil_5x4x3.ers", (5, 4, 3), 3, 172800.0, 2)])
def test_golden_files_read_and_rewrite(name, shape, b, t, k):
    with open(os.path.join(HERE, "golden", name), "rb") as f:
        text = f.read()
    edges, verts = restart.cartesian_counts(shape)
    n = int(np.prod(shape))
    st, pv, gm, out = restart.parse_restart(text, restart.info(edges, verts), n, b, blackoil=b == 3)
    assert st == 0, capi.load().gbfv_last_error()
    assert out.time == t and out.time_step_index == k and out.vtk_section == 1
    # written again from what was read: the same bytes
    again = restart.format_restart(restart.info(edges, verts, time=out.time, time_step_index=out.time_step_index),
                                   pv, gm)
    assert again == text


def test_every_double_reads_back_to_its_bits():
    rng = np.random.default_rng(3)
    special = [0.0, -0.0, 1e-310, -5e-324, 1.7976931348623157e308, 0.1, 1.0 / 3.0, 2.0 ** -1074, 123456789.123456789]
    vals = np.concatenate([special, rng.standard_normal(3000) * 10.0 ** rng.integers(-300, 300, 3000)])
    pv = vals[: len(vals) // 3 * 3].reshape(-1, 3)
    gm = rng.integers(0, 3, len(pv)).astype(np.int32)
    inf = restart.info(10, 20, time=np.nextafter(86400.0, 1e9))
    text = restart.format_restart(inf, pv, gm)
    st, pv2, gm2, out = restart.parse_restart(text, inf, len(pv), 3, blackoil=True)
    assert st == 0
    assert np.array_equal(pv.view(np.int64), pv2.view(np.int64))
    assert np.array_equal(gm, gm2) and out.time == inf.time


def test_malformed_files_are_rejected():
    pv, gm, shape = _oracle_state("blackoil")
    edges, verts = restart.cartesian_counts(shape)
    inf = restart.info(edges, verts)
    text = restart.format_restart(inf, pv, gm)
    n = len(pv)
    lib = capi.load()
    # another grid (cookie mismatch)
    assert restart.parse_restart(text, restart.info(edges + 1, verts), n, 3, True)[0] == capi.ERR_ARG
    assert b"cookie" in lib.gbfv_last_error()
    # fewer cells than the file has: unread values at the end of the section
    assert restart.parse_restart(text, inf, n - 1, 3, True)[0] == capi.ERR_ARG
    # truncated inside the entity section
    assert restart.parse_restart(text[: len(text) // 2], inf, n, 3, True)[0] == capi.ERR_ARG
    # a water meaning other than Sw is not a state of this model
    lines = text.split(b"\n")
    i = lines.index(b"Entities: Codim 0") + 1
    f = lines[i].split(b" ")
    f[4] = b"1"
    lines[i] = b" ".join(f)
    assert restart.parse_restart(b"\n".join(lines), inf, n, 3, True)[0] == capi.ERR_UNSUPPORTED


@pytest.mark.parametrize("field,value,want", [
    (3, b"3", capi.ERR_UNSUPPORTED),   # gas meaning Disabled: valid in the reference, not in this model
    (3, b"7", capi.ERR_ARG),           # no such gas meaning
    (3, b"1.5", capi.ERR_ARG),
    (3, b"nan", capi.ERR_ARG),
    (5, b"3", capi.ERR_ARG),           # no such pressure meaning
    (6, b"-1", capi.ERR_ARG),          # negative PVT region
    (6, b"1", capi.ERR_UNSUPPORTED),   # a second PVT region
])
def test_entity_meanings_are_checked_integers(field, value, want):
    pv, gm, shape = _oracle_state("blackoil")
    edges, verts = restart.cartesian_counts(shape)
    inf = restart.info(edges, verts)
    lines = restart.format_restart(inf, pv, gm).split(b"\n")
    i = lines.index(b"Entities: Codim 0") + 1
    f = lines[i].split(b" ")
    f[field] = value
    lines[i] = b" ".join(f)
    assert restart.parse_restart(b"\n".join(lines), inf, len(pv), 3, True)[0] == want


@pytest.mark.parametrize("line,field,value", [(0, 0, b"1e300"), (0, 5, b"2.5"), (0, 0, b"nan"),
                                              (2, 0, b"nan"), (3, 0, b"nan"), (3, 0, b"1e300"), (3, 0, b"-1")])
def test_simulator_and_vtk_integers_are_checked(line, field, value):
    """Episode and time-step indices, the writer count and the meta file's
    length must be integers in range; a bare conversion of NaN or 1e300 to
    an integer (or a byte offset) is undefined."""
    pv, gm, shape = _oracle_state("blackoil")
    edges, verts = restart.cartesian_counts(shape)
    inf = restart.info(edges, verts)
    inf.vtk_section, inf.vtk_writer_num = 1, 2
    lines = restart.format_restart(inf, pv, gm).split(b"\n")
    base = lines.index(b"Simulator") + 1   # the Simulator values; +2: writer count, +3: meta length
    k = base + line
    f = lines[k].split(b" ")
    f[field] = value
    lines[k] = b" ".join(f)
    assert restart.parse_restart(b"\n".join(lines), inf, len(pv), 3, True)[0] == capi.ERR_ARG


@pytest.mark.parametrize("d,name,t,r", [(".", "lens", 0.0, 0), ("", "lens", 1000.0, 0), ("out", "res", 86400.0, 1),
                                        ("out/", "res", 12.5, 0), ("a/b", "x", 3.1536e7, 3),
                                        (None, "y", 1e-3, 0)])
def test_file_names(d, name, t, r):
    assert restart.restart_file_name(d, name, t, r) == R.file_name(d, name, t, r)


def test_large_state_formatted_and_parsed_by_threads():
    # above 65536 cells the text is formatted and parsed in parallel ranges
    rng = np.random.default_rng(11)
    n = 100003
    pv = rng.standard_normal((n, 3)) * np.array([1e7, 1.0, 1e2])
    gm = rng.integers(0, 3, n).astype(np.int32)
    inf = restart.info(7, 9, time=5.0)
    text = restart.format_restart(inf, pv, gm)
    assert text == R.format_restart(pv, gm, num_edges=7, num_vertices=9, time=5.0)
    st, pv2, gm2, _ = restart.parse_restart(text, inf, n, 3, blackoil=True)
    assert st == 0 and np.array_equal(pv, pv2) and np.array_equal(gm, gm2)


def test_vertex_centred_entities_are_the_vertices():
    """A vertex-centred state (VcfvDiscretization::serialize writes the
    entities of codimension dim): the section names codim 2, the cookie the
    element count, one line per vertex; parsed back bit for bit."""
    prob = problems.lens_vcfv(12, 8)
    orc = O.Oracle(prob, capi.default_params(linear_tolerance=1e-6))
    assert orc.time_integration(2, 250.0)[0] == 0
    x, _ = orc.solution()
    pv = x.reshape(-1, 2)
    edges, verts = restart.cartesian_counts((12, 8))
    inf = restart.info(edges, verts, time=500.0, time_step_index=2, entity_codim=2, num_elements=96)
    got = restart.format_restart(inf, pv)
    want = R.format_restart(pv, num_edges=edges, num_vertices=verts, time=500.0, time_step_index=2,
                            entity_codim=2, num_elements=96)
    assert got == want
    assert b"numElements=96 " in got and b"\nEntities: Codim 2\n" in got
    st, back, _, out = restart.parse_restart(got, inf, len(pv), 2)
    assert st == 0 and np.array_equal(back, pv) and out.time == 500.0
    # a file of the cells' entities is not the vertices' file
    st0, *_ = restart.parse_restart(got, restart.info(edges, verts), len(pv), 2)
    assert st0 != 0
