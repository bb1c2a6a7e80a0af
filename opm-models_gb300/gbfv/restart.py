"""Restart files in the reference's text format (Opm::Restart,
opm/models/io/restart.hh; written by Simulator::serialize, simulator.hh:
906-962), through the C ABI: format/parse a state held on the host, and
write/read a context's device state (Context.write_restart/read_restart)."""
import ctypes as C

import numpy as np

from . import capi


def info(num_edges, num_vertices, time=0.0, time_step_index=0, episode_index=0, episode_start_time=0.0,
         episode_length=0.0, start_time=0.0, vtk_section=True, vtk_writer_num=0, num_cpus=1, rank=0,
         entity_codim=0, num_elements=0):
    """gbfv_restart_info for a grid with the given edge and vertex counts
    (gridView.size(dim-1), gridView.size(dim)) and the Simulator's clock;
    entity_codim / num_elements for the vertices of a vertex-centred grid
    (a context sets both itself when it writes or reads)."""
    return capi.RestartInfo(num_cpus, rank, num_edges, num_vertices, episode_index, time_step_index,
                            episode_start_time, episode_length, start_time, time, 1 if vtk_section else 0,
                            vtk_writer_num, entity_codim, num_elements)


def cartesian_counts(shape):
    """(edges, vertices) of a structured grid of `shape` cells (2D or 3D):
    entities of codimension dim-1 and dim, as a YaspGrid counts them."""
    if len(shape) == 2:
        nx, ny = shape
        return nx * (ny + 1) + (nx + 1) * ny, (nx + 1) * (ny + 1)
    nx, ny, nz = shape
    edges = nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz
    return edges, (nx + 1) * (ny + 1) * (nz + 1)


def format_restart(inf, pv, gas_meaning=None):
    """The file's text (bytes) for primary variables pv [num_cells, b]."""
    lib = capi.load()
    pv = np.ascontiguousarray(pv, dtype=np.float64)
    n, b = pv.shape
    gm = None if gas_meaning is None else np.ascontiguousarray(gas_meaning, dtype=np.int32)
    size = C.c_size_t(0)
    capi.check(lib.gbfv_format_restart(C.byref(inf), n, b, capi.as_ptr(pv, C.c_double), capi.as_ptr(gm, C.c_int32),
                                       None, 0, C.byref(size)), "gbfv_format_restart")
    buf = C.create_string_buffer(size.value)
    capi.check(lib.gbfv_format_restart(C.byref(inf), n, b, capi.as_ptr(pv, C.c_double), capi.as_ptr(gm, C.c_int32),
                                       buf, size.value, C.byref(size)), "gbfv_format_restart")
    return buf.raw[:size.value]


def parse_restart(text, expect, num_cells, b, blackoil=False):
    """(pv [num_cells, b], gas meanings or None, RestartInfo) read from text;
    returns (status, ...) so malformed files can be checked."""
    lib = capi.load()
    pv = np.zeros((num_cells, b))
    gm = np.zeros(num_cells, np.int32) if blackoil else None
    out = capi.RestartInfo()
    st = lib.gbfv_parse_restart(text, len(text), C.byref(expect), num_cells, b, capi.as_ptr(pv, C.c_double),
                                capi.as_ptr(gm, C.c_int32), C.byref(out))
    return st, pv, gm, out


def restart_file_name(output_dir, sim_name, time, rank=0):
    lib = capi.load()
    buf = C.create_string_buffer(4096)
    capi.check(lib.gbfv_restart_file_name(None if output_dir is None else output_dir.encode(), sim_name.encode(),
                                          float(time), rank, buf, len(buf)), "gbfv_restart_file_name")
    return buf.value.decode()
