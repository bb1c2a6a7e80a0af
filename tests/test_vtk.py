"""VTK output (gbfv_write_vtk, gbfv_write_pvd, gbfv_output_fields): the
reference's VtkMultiWriter time series with its multi-phase and
primary-variable modules (opm/models/io/vtkmultiwriter.hh:64-540,
vtkmultiphasemodule.hh:84-460, vtkprimaryvarsmodule.hh:54-170).

CPU: file names (<sim>-<5 digits>.vtu), the .pvd collection, the
structured grid's vertices in VTK order, and the oracle's output fields
(saturations sum to one, mobility = relative permeability / viscosity).
GPU: the device's output fields equal the oracle's at the same state, and a
written .vtu parses as XML with the reference's field names in the modules'
order, float-rounded values equal to the oracle's, the grid's points and
cells; the .pvd lists every file with its time."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import oracle as O
from gbfv import Context, capi, problems
from gbfv import vtk


def test_file_names_and_collection(built, tmp_path):
    assert vtk.file_name("lens", 0) == "lens-00000.vtu"
    assert vtk.file_name("lens", 123) == "lens-00123.vtu"
    assert vtk.file_name("", 7) == "sim-00007.vtu"
    import ctypes as C
    lib = capi.load()
    path = str(tmp_path / "lens.pvd")
    files = (C.c_char_p * 2)(b"lens-00000.vtu", b"lens-00001.vtu")
    times = (C.c_double * 2)(0.0, 250.125)
    assert lib.gbfv_write_pvd(path.encode(), 2, times, files) == 0
    root = ET.parse(path).getroot()
    assert root.get("type") == "Collection"
    ds = root.find("Collection").findall("DataSet")
    assert [(d.get("timestep"), d.get("file")) for d in ds] == [("0", "lens-00000.vtu"), ("250.125", "lens-00001.vtu")]


def test_structured_points_in_vtk_order():
    p = problems.lens(4, 3)
    pts, cells = vtk.structured_points(p)
    assert pts.shape == (20, 3) and cells.shape == (12, 4)
    # cell 0: (0,0), (1,0), (1,1), (0,1) counter-clockwise; its centre is the cell centre
    c0 = pts[cells[0]]
    assert np.allclose(c0[:, :2], [[0, 0], [1.5, 0], [1.5, 4 / 3], [0, 4 / 3]])
    assert np.allclose(pts[cells].mean(1), p.center.reshape(-1, 3))
    b = problems.blackoil(3, 2, 2)
    pts3, cells3 = vtk.structured_points(b)
    assert pts3.shape == (4 * 3 * 3, 3) and cells3.shape == (12, 8)
    assert np.allclose(pts3[cells3].mean(1), b.center.reshape(-1, 3))


def test_oracle_output_fields_are_consistent():
    for prob in (problems.lens(8, 6), problems.blackoil(5, 4, 3)):
        orc = O.Oracle(prob, capi.default_params())
        f = orc.output_fields()
        orc.close()
        nph = 2 if prob.b == 2 else 3
        assert np.allclose(f[6:6 + nph].sum(0), 1.0)
        assert np.all(f[12:12 + nph] >= 0.0) and np.all(f[12:12 + nph] <= 1.0)
        assert np.allclose(f[9:9 + nph], f[12:12 + nph] / f[15:15 + nph])
        assert np.array_equal(f[18], prob.porosity)


def _cell_arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid").find("Piece")
    cd = piece.find("CellData")
    arrays = [(a.get("Name"), np.array(a.text.split(), np.float32)) for a in cd.findall("DataArray")]
    pts = np.array(piece.find("Points").find("DataArray").text.split(), np.float32).reshape(-1, 3)
    cells = {a.get("Name"): np.array(a.text.split(), np.int64) for a in piece.find("Cells").findall("DataArray")}
    return piece, arrays, pts, cells


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["lens", "blackoil"])
def test_vtk_output_equals_the_oracle(built, tmp_path, kind):
    if kind == "lens":
        prob, dt, steps = problems.lens(24, 16), 250.0, 4
        names = ["PV_pressure_w", "PV_saturation_w", "DOF index"]
        phases = ["w", "n"]
    else:
        prob, dt, steps = problems.blackoil(10, 8, 4), 86400.0, 2
        names = ["PV_water_switching", "PV_pressure_switching", "PV_composition_switching", "DOF index"]
        phases = ["water", "oil", "gas"]
    for q in ("pressure", "density", "saturation", "mobility", "relativePerm", "viscosity"):
        names += ["%s_%s" % (q, ph) for ph in phases]
    names.append("porosity")
    prm = capi.default_params(linear_tolerance=1e-6)
    ctx = Context(prob, prm)
    w = vtk.MultiWriter(prob, str(tmp_path), kind, fields=511)
    w.write(ctx, 0.0)
    st, _, _, _, _ = ctx.time_integration(steps, dt, fixed_dt=True)
    assert st == 0
    path = w.write(ctx, steps * dt)
    x, m = ctx.solution()
    dev = vtk.output_fields(ctx)
    ctx.close()
    orc = O.Oracle(prob, prm)
    orc.set_solution(x, m)
    ref = orc.output_fields()
    orc.close()
    nph = len(phases)
    planes = [3 * k + a for k in range(6) for a in range(nph)] + [18]
    scale = np.maximum(np.abs(ref[planes]), 1e-300)
    assert np.max(np.abs(dev[planes] - ref[planes]) / scale) <= 1e-12
    piece, arrays, pts, cells = _cell_arrays(path)
    assert int(piece.get("NumberOfCells")) == prob.num_cells
    assert [a[0] for a in arrays] == names
    expect = [x.reshape(-1, prob.b)[:, e] for e in range(prob.b)] + [np.arange(prob.num_cells)]
    expect += [ref[p] for p in planes]
    for (name, got), want in zip(arrays, expect):
        assert np.array_equal(got, np.asarray(want).astype(np.float32)), name
    vp, vc = vtk.structured_points(prob)
    assert np.array_equal(pts, vp.astype(np.float32))
    assert np.array_equal(cells["connectivity"], vc.ravel())
    assert np.array_equal(cells["offsets"], vc.shape[1] * np.arange(1, prob.num_cells + 1))
    assert set(cells["types"].tolist()) == {9 if prob.b == 2 else 12}
    coll = ET.parse(os.path.join(str(tmp_path), kind + ".pvd")).getroot().find("Collection")
    assert [d.get("file") for d in coll.findall("DataSet")] == [kind + "-00000.vtu", kind + "-00001.vtu"]


def test_vertex_centred_points_and_cells():
    """A vertex-centred grid: the points are its degrees of freedom, the
    cells its elements in VTK's counter-clockwise corner order."""
    p = problems.lens_vcfv(4, 3)
    pts, cells = vtk.structured_points(p)
    assert pts.shape == (20, 3) and cells.shape == (12, 4)
    assert np.allclose(pts[cells[0]][:, :2], [[0, 0], [1.5, 0], [1.5, 4 / 3], [0, 4 / 3]])
    assert np.array_equal(pts, p.center.reshape(-1, 3))


@pytest.mark.gpu
def test_vertex_centred_vtk_output_is_vertex_data(built, tmp_path):
    """VcfvBaseOutputModule writes vertex data: the fields of the vertex-
    centred lens as PointData over the vertices, the elements as cells, the
    values the oracle's output quantities rounded to float."""
    prob = problems.lens_vcfv(12, 8)
    prm = capi.default_params(linear_tolerance=1e-8)
    ctx = Context(prob, prm)
    st, *_ = ctx.time_integration(3, 250.0)
    assert st == 0
    w = vtk.MultiWriter(prob, str(tmp_path), "lensvcfv", fields=vtk.DEFAULT_FIELDS | vtk.PRIMARY_VARS)
    path = w.write(ctx, 750.0)
    x, m = ctx.solution()
    ctx.close()
    orc = O.Oracle(prob, prm)
    orc.set_solution(x, m)
    ref = orc.output_fields()
    orc.close()
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid").find("Piece")
    assert piece.find("CellData") is None
    pd = piece.find("PointData")
    arrays = [(a.get("Name"), np.array(a.text.split(), np.float32)) for a in pd.findall("DataArray")]
    assert int(piece.get("NumberOfPoints")) == prob.num_cells
    assert int(piece.get("NumberOfCells")) == len(prob.elem_corner) // 4
    names = [a[0] for a in arrays]
    assert names[:2] == ["PV_pressure_w", "PV_saturation_w"]
    got = dict(arrays)
    assert np.allclose(got["PV_saturation_w"], x.reshape(-1, 2)[:, 1].astype(np.float32), rtol=0, atol=0)
    for q, k in (("pressure", 0), ("density", 1), ("saturation", 2), ("relativePerm", 4)):
        for a, ph in enumerate(("w", "n")):
            want = ref[3 * k + a].astype(np.float32)
            assert np.max(np.abs(got["%s_%s" % (q, ph)] - want)) <= 1e-6 * max(1.0, np.max(np.abs(want))), q
    cells = {a.get("Name"): np.array(a.text.split(), np.int64) for a in piece.find("Cells").findall("DataArray")}
    _, vc = vtk.structured_points(prob)
    assert np.array_equal(cells["connectivity"], vc.ravel())
