"""Failure detection on the GPU without a fault: a device-side wait that
nothing completes gives up after its bound and reports GBFV_ERR_TIMEOUT; the
device stays usable for the next solve."""
import ctypes as C

import pytest

from gbfv import Context, capi, problems

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_device_stays_usable(built):
    lib = capi.load()
    ms = C.c_double()
    st = lib.gbfv_selftest_wait_timeout(C.byref(ms))
    assert st == capi.ERR_TIMEOUT
    assert 0.0 < ms.value < 5000.0
    ctx = Context(problems.lens(nx=12, ny=8), capi.default_params(linear_tolerance=1e-6))
    rep_st, *_ = ctx.time_integration(2, 250.0)
    assert rep_st == 0
