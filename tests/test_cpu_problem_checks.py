"""CPU checks of the problem-description validation that gbfv_create runs
before it looks for a GPU: every inconsistent count, offset, enum field or
PVT table is GBFV_ERR_ARG, with a message, and the descriptions the problem
builders make (every variant the GPU tests, smoke() and bench.py create)
pass it -- without a GPU they then stop at GBFV_ERR_NO_DEVICE.  The
stand-alone linear solver checks its row pointers and column indices the
same way."""
import copy
import ctypes as C

import numpy as np
import pytest

from gbfv import capi, problems


def _status(p, tweak=None):
    """gbfv_create's status for problem data p; tweak(struct) edits the C
    struct (pointer fields) before the call."""
    lib = capi.load()
    s = p.struct()
    if tweak:
        tweak(s)
    st = C.c_int(-1)
    prm = capi.default_params()
    h = lib.gbfv_create(C.byref(s), C.byref(prm), C.byref(st))
    if h:
        lib.gbfv_destroy(h)
    return st.value, lib.gbfv_last_error().decode()


VALID = [
    lambda: problems.lens(),
    lambda: problems.lens(nx=1, ny=2),
    lambda: problems.lens(nx=1, ny=2, flux="trans"),
    lambda: problems.lens(law="bc"),
    lambda: problems.lens(flux="trans"),
    lambda: problems.lens(nx=16, ny=10, dim=3, nz=6, flux="darcy"),
    lambda: problems.lens(nx=16, ny=10, dim=3, nz=6, flux="trans"),
    lambda: problems.tiny_lens(6, 4),
    lambda: problems.blackoil(4, 3, 2),
    lambda: problems.blackoil(9, 11, 4, seed=15),
    lambda: problems.blackoil(40, 36, 8, seed=9),
    lambda: problems.blackoil(100, 100, 20),
    lambda: problems.ensemble_member(8, 1, 1.0),
    lambda: problems.ensemble_member(3000, 7, 2.0),
]


@pytest.mark.parametrize("make", VALID)
def test_builder_descriptions_pass(built, make):
    st, msg = _status(make())
    assert st in (capi.OK, capi.ERR_NO_DEVICE), (st, msg)


def _edit(p, field, fn):
    q = copy.deepcopy(p)
    a = np.array(getattr(q, field), copy=True)
    fn(a)
    setattr(q, field, a)
    return q


def _replace(p, field, value):
    q = copy.deepcopy(p)
    setattr(q, field, value)
    return q


def _set(i, v):
    def f(a):
        a[i] = v
    return f


LENS = problems.lens(nx=6, ny=4)
BLACKOIL = problems.blackoil(4, 3, 2)
assert len(BLACKOIL.constraint_meaning) > 0     # the corner wells are constraint rows


@pytest.mark.parametrize("name,p", [
    ("conn_ptr starts above 0", _edit(LENS, "conn_ptr", _set(0, 1))),
    ("conn_ptr decreases", _edit(LENS, "conn_ptr", _set(3, 0))),
    ("conn_ptr ends past num_conn", _edit(LENS, "conn_ptr", _set(-1, 10 ** 6))),
    ("bface_ptr decreases", _edit(LENS, "bface_ptr", _set(2, -5))),
    ("bface_ptr ends short", _edit(LENS, "bface_ptr", _set(-1, 1))),
    ("unknown boundary type", _edit(LENS, "bface_type", _set(0, 7))),
    ("material index = num_materials", _edit(LENS, "material", _set(0, 2))),
    ("negative material index", _edit(LENS, "material", _set(5, -1))),
    ("unknown law", _edit(LENS, "material_params", _set(0, 5.0))),
    ("NaN law", _edit(LENS, "material_params", _set(0, np.nan))),
    ("fractional law", _edit(LENS, "material_params", _set(0, 0.5))),
    ("three-phase law in the immiscible model", _edit(LENS, "material_params", _set(0, capi.LAW_COREY3P))),
    ("no materials", _replace(LENS, "material_params", np.zeros(0))),
    ("constraint row = num_constraints", _edit(BLACKOIL, "constraint", _set(0, len(BLACKOIL.constraint_meaning)))),
    ("constraint row below -1", _edit(BLACKOIL, "constraint", _set(1, -2))),
    ("unknown constraint gas meaning", _edit(BLACKOIL, "constraint_meaning", _set(0, 3))),
])
def test_inconsistent_arrays_are_rejected(built, name, p):
    st, msg = _status(p)
    assert st == capi.ERR_ARG, (name, st, msg)
    assert "problem description" in msg, msg


def _pvt_edit(key, fn):
    q = copy.deepcopy(BLACKOIL)
    a = dict(q.pvt_arrays)
    a[key] = np.array(a[key], copy=True)
    fn(a[key])
    q.pvt_arrays = a
    return q


@pytest.mark.parametrize("name,p", [
    ("oil pressures not increasing", _pvt_edit("oil_p", _set(2, 0.0))),
    ("flat R_s step", _pvt_edit("oil_rs", lambda a: a.__setitem__(3, a[2]))),
    ("NaN gas pressure", _pvt_edit("gas_p", _set(1, np.nan))),
    ("zero B_o", _pvt_edit("oil_bo", _set(0, 0.0))),
    ("negative B_g", _pvt_edit("gas_bg", _set(4, -1.0))),
])
def test_inconsistent_pvt_tables_are_rejected(built, name, p):
    st, msg = _status(p)
    assert st == capi.ERR_ARG, (name, st, msg)
    assert "PVT" in msg, msg


def _null(field):
    def f(s):
        setattr(s, field, None)
    return f


@pytest.mark.parametrize("name,p,tweak", [
    ("NULL centres", LENS, _null("center")),
    ("NULL conn_ptr", LENS, _null("conn_ptr")),
    ("NULL boundary values with free-flow faces", LENS, _null("bface_value")),
    ("NULL boundary normals", LENS, _null("bface_normal")),
    ("NULL material parameters", LENS, _null("material_params")),
    ("NULL constraint table", BLACKOIL, _null("constraint_pv")),
    ("NULL PVT", BLACKOIL, _null("pvt")),
    ("unknown model", LENS, lambda s: setattr(s, "model", 5)),
    ("unknown flux module", LENS, lambda s: setattr(s, "flux_module", 3)),
    ("no cells", LENS, lambda s: setattr(s, "num_cells", 0)),
    ("negative num_conn", LENS, lambda s: setattr(s, "num_conn", -1)),
    ("PVT table of one row", BLACKOIL, lambda s: setattr(s.pvt.contents, "n_oil", 1)),
    ("PVT column NULL", BLACKOIL, lambda s: setattr(s.pvt.contents, "gas_mu", None)),
])
def test_inconsistent_struct_fields_are_rejected(built, name, p, tweak):
    st, msg = _status(p, tweak)
    assert st == capi.ERR_ARG, (name, st, msg)
    assert "problem description" in msg, msg


def test_no_flow_only_boundaries_need_no_boundary_values(built):
    p = problems.lens(nx=6, ny=4)
    p.bface_type = np.zeros_like(p.bface_type)
    st, msg = _status(p, _null("bface_value"))
    assert st in (capi.OK, capi.ERR_NO_DEVICE), (st, msg)


def _linsolver_status(rp, col, n=None):
    lib = capi.load()
    rp = np.ascontiguousarray(rp, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    st = C.c_int(-1)
    prm = capi.default_params()
    h = lib.gbfv_linsolver_create(len(rp) - 1 if n is None else n, 3, capi.as_ptr(rp, C.c_int32),
                                  capi.as_ptr(col, C.c_int32), C.byref(prm), C.byref(st))
    if h:
        lib.gbfv_linsolver_destroy(h)
    return st.value, lib.gbfv_last_error().decode()


# a 1D three-point pattern of 4 block rows
RP = [0, 2, 5, 8, 10]
COL = [0, 1, 0, 1, 2, 1, 2, 3, 2, 3]


@pytest.mark.parametrize("name,rp,col", [
    ("row_ptr starts above 0", [1, 2, 5, 8, 10], COL),
    ("row_ptr decreases", [0, 2, 1, 8, 10], COL),
    ("negative column", RP, [0, 1, 0, 1, 2, 1, 2, 3, 2, -3]),
    ("column past the last row", RP, [0, 1, 0, 1, 2, 1, 2, 4, 2, 3]),
])
def test_linear_solver_pattern_is_checked_before_device_work(built, name, rp, col):
    st, msg = _linsolver_status(rp, col)
    assert st == capi.ERR_ARG, (name, st, msg)


def test_linear_solver_valid_pattern_passes_the_checks(built):
    st, msg = _linsolver_status(RP, COL)
    assert st in (capi.OK, capi.ERR_NO_DEVICE), (st, msg)


@pytest.mark.parametrize("field,value", [("precision", 2), ("precision", -1), ("local_linearizer", 5),
                                         ("numeric_difference_method", 2)])
def test_enum_parameters_are_checked_by_every_create_call(built, field, value):
    lib = capi.load()
    prm = capi.default_params()
    setattr(prm, field, value)
    st = C.c_int(-1)
    s = LENS.struct()
    assert not lib.gbfv_create(C.byref(s), C.byref(prm), C.byref(st)) and st.value == capi.ERR_ARG
    rp = np.ascontiguousarray(RP, np.int32)
    col = np.ascontiguousarray(COL, np.int32)
    st.value = -1
    assert not lib.gbfv_linsolver_create(4, 3, capi.as_ptr(rp, C.c_int32), capi.as_ptr(col, C.c_int32),
                                         C.byref(prm), C.byref(st))
    assert st.value == capi.ERR_ARG
    st.value = -1
    assert not lib.gbfv_serve_create(2, capi.MODEL_IMMISCIBLE_2P, C.byref(prm), 0, 1000, C.byref(st))
    assert st.value == capi.ERR_ARG
    st.value = -1
    arr = (capi.Problem * 1)(s)
    assert not lib.gbfv_batch_create(arr, 1, C.byref(prm), 0, C.byref(st))
    assert st.value == capi.ERR_ARG
