"""VTK output of a context's state (gbfv_write_vtk / gbfv_write_pvd): the
reference's VtkMultiWriter time series (opm/models/io/vtkmultiwriter.hh:64-540)
-- one .vtu per time step named <sim>-<number>.vtu and the .pvd collection
that lists them."""
import ctypes as C
import os

import numpy as np

from . import capi

PRESSURE, DENSITY, SATURATION, MOBILITY, RELPERM, VISCOSITY, POROSITY, PRIMARY_VARS, DOF_INDEX = (
    1, 2, 4, 8, 16, 32, 64, 128, 256)
DEFAULT_FIELDS = PRESSURE | DENSITY | SATURATION | RELPERM | POROSITY


class VtkGrid(C.Structure):
    _fields_ = [("num_points", C.c_int32), ("points", C.POINTER(C.c_double)),
                ("vertices_per_cell", C.c_int32), ("cell_vertices", C.POINTER(C.c_int32)),
                ("num_cells", C.c_int32)]


def structured_points(problem):
    """Vertices and cells (VTK vertex order) of a problem built on
    problems.structured_grid: (points [P, 3], cells [N, 4 or 8]).  For a
    vertex-centred problem (problems.lens_vcfv) the points are its degrees
    of freedom and the cells its elements (corners 0, 1, 3, 2 of the
    reference element: counter-clockwise)."""
    if getattr(problem, "elem_corner", None) is not None:
        pts = np.ascontiguousarray(problem.center.reshape(-1, 3), float)
        cells = problem.elem_corner.reshape(-1, 4)[:, [0, 1, 3, 2]]
        return pts, np.ascontiguousarray(cells, np.int32)
    g = problem.grid
    nx, ny, dim = g["nx"], g["ny"], g["dim"]
    nz = g["nz"] if dim == 3 else 1
    hi = g["bbox_max"]
    xs = np.linspace(0.0, hi[0], nx + 1)
    ys = np.linspace(0.0, hi[1], ny + 1)
    if dim == 2:
        X, Y = np.meshgrid(xs, ys, indexing="xy")
        pts = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)
        i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
        i, j = i.ravel(), j.ravel()
        v = lambda a, b: a + (nx + 1) * b  # noqa: E731
        cells = np.stack([v(i, j), v(i + 1, j), v(i + 1, j + 1), v(i, j + 1)], 1)
    else:
        zs = np.linspace(0.0, hi[2], nz + 1)
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        v = lambda a, b, c: a + (nx + 1) * (b + (ny + 1) * c)  # noqa: E731
        cells = np.stack([v(i, j, k), v(i + 1, j, k), v(i + 1, j + 1, k), v(i, j + 1, k),
                          v(i, j, k + 1), v(i + 1, j, k + 1), v(i + 1, j + 1, k + 1), v(i, j + 1, k + 1)], 1)
    return np.ascontiguousarray(pts, float), np.ascontiguousarray(cells, np.int32)


def output_fields(ctx):
    """[19, N] output quantities of the context's current solution."""
    out = np.zeros(19 * ctx.N)
    capi.check(ctx.lib.gbfv_output_fields(ctx.h, out.ctypes.data_as(C.POINTER(C.c_double))), "gbfv_output_fields")
    return out.reshape(19, ctx.N)


def file_name(sim_name, writer_num):
    buf = C.create_string_buffer(512)
    capi.check(capi.load().gbfv_vtk_file_name(sim_name.encode(), writer_num, buf, 512), "gbfv_vtk_file_name")
    return buf.value.decode()


class MultiWriter:
    """A time series of VTK files: write(ctx, time) writes the next .vtu and
    rewrites the .pvd collection (VtkMultiWriter::beginWrite / endWrite)."""

    def __init__(self, problem, output_dir=".", sim_name="sim", fields=DEFAULT_FIELDS):
        self.pts, self.cells = structured_points(problem)
        vertex_data = getattr(problem, "elem_corner", None) is not None
        self.grid = VtkGrid(len(self.pts), self.pts.ctypes.data_as(C.POINTER(C.c_double)), self.cells.shape[1],
                            self.cells.ctypes.data_as(C.POINTER(C.c_int32)),
                            len(self.cells) if vertex_data else 0)
        self.dir, self.sim, self.fields = output_dir, sim_name or "sim", fields
        self.times, self.files = [], []

    def write(self, ctx, time):
        name = file_name(self.sim, len(self.files))
        capi.check(ctx.lib.gbfv_write_vtk(ctx.h, C.addressof(self.grid), self.fields,
                                          os.path.join(self.dir, name).encode()), "gbfv_write_vtk")
        self.times.append(float(time))
        self.files.append(name)
        n = len(self.files)
        arr = (C.c_char_p * n)(*[f.encode() for f in self.files])
        tm = (C.c_double * n)(*self.times)
        capi.check(capi.load().gbfv_write_pvd(os.path.join(self.dir, self.sim + ".pvd").encode(), n, tm, arr),
                   "gbfv_write_pvd")
        return os.path.join(self.dir, name)
