"""CPU checks of the drop-in boundary: the C-ABI library builds, loads and
exports every entry point include/gbfv.h declares; the ctypes mirrors of
the C structs have the C layout; host-side logic (problem builders,
parameter defaults) matches the reference's."""
import ctypes as C
import os
import subprocess

import numpy as np

from gbfv import capi, problems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol(built):
    lib = C.CDLL(capi.LIB_PATH)
    names = capi.exported_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "gbfv.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(gbfv_problem),"
        " sizeof(gbfv_params), sizeof(gbfv_blackoil_pvt), sizeof(gbfv_newton_report),"
        " sizeof(gbfv_kernel_stats), offsetof(gbfv_problem, pvt), offsetof(gbfv_params, max_time_step_divisions));"
        " return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    got = [int(v) for v in out]
    want = [C.sizeof(capi.Problem), C.sizeof(capi.Params), C.sizeof(capi.BlackOilPvt),
            C.sizeof(capi.NewtonReport), C.sizeof(capi.KernelStats), capi.Problem.pvt.offset,
            capi.Params.max_time_step_divisions.offset]
    assert got == want


def test_reference_parameter_defaults():
    p = capi.default_params()
    # newtonmethodparameters.hh:31-53, linalgparameters.hh:41-78,
    # blackoilnewtonmethodparameters.hh
    assert p.newton_tolerance == 1e-8 and p.newton_max_iterations == 20
    assert p.newton_target_iterations == 10 and p.newton_max_error == 1e100
    assert p.linear_tolerance == 1e-3 and p.linear_abs_tolerance == -1.0
    assert p.linear_max_iterations == 1000 and p.linear_max_error == 1e7
    assert p.dp_max_rel == 0.3 and p.ds_max == 0.2 and p.pv_oscillation_threshold == 1e-5
    assert p.max_time_step_divisions == 10


def test_lens_geometry_matches_reference_problem():
    p = problems.lens()
    assert p.num_cells == 48 * 32
    assert len(p.conn_nbr) == 2 * (47 * 32 + 48 * 31)
    assert len(p.bface_area) == 2 * (48 + 32)
    assert int((p.bface_type == capi.BC_MASSRATE).sum()) == 8      # inlet x in (2,3) m
    assert int((p.bface_type == capi.BC_FREEFLOW).sum()) == 64     # left + right
    assert int(p.material.sum()) == 24 * 8                         # lens [1,4]x[2,3] m
    pv = p.init_pv.reshape(-1, 2)
    assert np.all(pv[:, 1] == 1.0)
    # hydrostatic initial pressure (lensproblem.hh:549-582)
    depth = 4.0 - p.center.reshape(-1, 3)[:, 1]
    assert np.allclose(pv[:, 0], 1e5 + 1000.0 * 9.81 * depth)


def test_blackoil_builder_wells_and_tables():
    p = problems.blackoil(10, 8, 3)
    cons = p.constraint
    assert int((cons == 0).sum()) == 3 and int((cons == 1).sum()) == 3
    t = p.pvt_arrays
    assert len(t["oil_p"]) == 10 and np.all(np.diff(t["oil_rs"]) > 0)
    k = p.perm.reshape(-1, 3)
    assert np.allclose(k[:, 2], 0.1 * k[:, 0])
    assert p.porosity.min() >= 0.15 and p.porosity.max() <= 0.30


def test_footprint_estimate_is_monotone(built):
    lib = capi.load()
    f = lib.gbfv_footprint_bytes
    a, b = f(100000, 3, 3), f(200000, 3, 3)
    assert 0 < a < b and b - a > 100000 * 1000       # at least 1 KB per cell of a 3x3 system
    assert f(100000, 2, 3) < a                         # 2x2 blocks take less
    assert f(0, 3, 3) == -1 and f(10, 4, 3) == -1      # rejected arguments


def test_sizes_beyond_32bit_device_indexing_are_rejected_before_device_work(built):
    """GBFV_MAX_CELLS: every create entry point turns a size whose device
    indices would not fit 32 bits into GBFV_ERR_UNSUPPORTED before it reads
    the arrays or looks for a device, so this runs without a GPU."""
    import re
    with open(os.path.join(ROOT, "include", "gbfv.h")) as f:
        m = re.search(r"#define GBFV_MAX_CELLS (\d+)", f.read())
    assert m and int(m.group(1)) == capi.MAX_CELLS
    ld = (capi.MAX_CELLS + 63) // 64 * 64
    assert ld == capi.MAX_CELLS and 64 * ld <= 2**31 - 1 < 64 * (ld + 64)
    lib = capi.load()
    st = C.c_int(-1)
    prob = problems.blackoil(4, 4, 2)
    s = prob.struct()
    s.num_cells = capi.MAX_CELLS + 1
    prm = capi.default_params()
    assert not lib.gbfv_create(C.byref(s), C.byref(prm), C.byref(st))
    assert st.value == capi.ERR_UNSUPPORTED
    rp = np.zeros(2, np.int32)
    col = np.zeros(1, np.int32)
    st.value = -1
    assert not lib.gbfv_linsolver_create(capi.MAX_CELLS + 1, 3, rp.ctypes.data_as(C.POINTER(C.c_int32)),
                                         col.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(prm), C.byref(st))
    assert st.value == capi.ERR_UNSUPPORTED
    st.value = -1
    assert not lib.gbfv_serve_create(4, capi.MODEL_BLACKOIL_3P, C.byref(prm), 0, capi.MAX_CELLS + 1, C.byref(st))
    assert st.value == capi.ERR_UNSUPPORTED
    f = lib.gbfv_footprint_bytes
    assert f(capi.MAX_CELLS, 3, 3) > 0 and f(capi.MAX_CELLS + 1, 3, 3) == -1


CTYPES_BINDING = """
import ctypes as C
lib = C.CDLL("opm-models_gb300/_build/libgbfv.so")
lib.gbfv_create.restype = C.c_void_p
lib.gbfv_create.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
lib.gbfv_linearize.argtypes = [C.c_void_p]
lib.gbfv_newton_apply.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
lib.gbfv_last_error.restype = C.c_char_p
"""


def test_ctypes_binding_runs(built):
    """The ctypes binding a Python host adds (the library path relative to
    the repository root) loads the library and binds its entry points."""
    import sys
    r = subprocess.run([sys.executable, "-c", CTYPES_BINDING], cwd=ROOT, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr


def test_batch_report_sizes_its_arrays_from_the_step_count():
    """Batch.report asks for the step count first (NULL arrays) and then
    reads exactly that many steps, however many there are."""
    import gbfv

    class FakeLib:
        def __init__(self, steps):
            self.steps, self.calls = steps, []

        def gbfv_batch_system_report(self, h, i, st, n, sdt, sn, sl, nl):
            self.calls.append(sdt is None)
            n._obj.value = self.steps
            if sdt is not None:
                for k in range(self.steps):
                    sdt[k], sn[k], sl[k] = 0.5 * k, k % 7, 3 * k
                st._obj.value, nl._obj.value = 0, self.steps + 2
            return 0

    for steps in (0, 3, 5000):
        b = object.__new__(gbfv.Batch)
        b.lib, b.h = FakeLib(steps), 1
        st, sdt, sn, sl, nl = b.report(0)
        assert b.lib.calls == [True, False]
        assert st == 0 and nl == steps + 2 and len(sdt) == len(sn) == len(sl) == steps
        assert np.array_equal(sdt, 0.5 * np.arange(steps)) and np.array_equal(sl, 3 * np.arange(steps))
        b.h = None
