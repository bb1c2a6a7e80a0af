"""GPU checks of gbfv_newton_error_noalloc, the allocation-free Newton error.

It is called through the C ABI on a residual held in device memory and
compared with gbfv_newton_error of a context on the same residual (the
maximum is order independent, so the two agree exactly), twice in a row.
This file is collected last so that it also runs after the other GPU tests
in one process; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

from gbfv import Context, capi, problems

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 24  # GBFV_NOALLOC_MAX_CELLS


def _fn():
    lib = capi.load()
    f = lib.gbfv_newton_error_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_double)]
    return lib, f


def _call(f, d_res, d_skip, n, b, stream=None):
    err = C.c_double(-1.0)
    st = f(d_res, d_skip, n, b, stream, C.byref(err))
    return st, err.value


def _device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("which", ["lens", "blackoil"])
def test_noalloc_matches_context_newton_error(built, which):
    import torch
    if which == "lens":
        prob, dt, steps = problems.lens(), 250.0, 3
    else:
        prob, dt, steps = problems.blackoil(24, 20, 6), 86400.0, 2
    prm = capi.default_params(linear_tolerance=1e-6)
    ctx = Context(prob, prm)
    assert ctx.time_integration(steps, dt)[0] == 0
    assert ctx.linearize(dt, 0) == 0
    assert ctx.linearize(dt, 1) == 0
    st, ref = ctx.newton_error()
    assert st == 0 and ref > 0.0
    res = ctx.residual()
    skip = (np.asarray(prob.constraint) >= 0).astype(np.int32)
    d_res, d_skip = _device(res), _device(skip)
    torch.cuda.synchronize()
    _, f = _fn()
    stream = torch.cuda.Stream()
    for _ in range(2):  # two calls in a row give the same answer
        st, err = _call(f, d_res.data_ptr(), d_skip.data_ptr(), ctx.N, ctx.b, stream.cuda_stream)
        assert st == 0, capi.load().gbfv_last_error().decode()
        assert err == ref, (err, ref)
    # without skip flags the constraint cells count too (their residual is 0)
    st, err = _call(f, d_res.data_ptr(), None, ctx.N, ctx.b)
    assert st == 0 and err == max(ref, float(np.abs(res).max()))


def test_noalloc_ragged_sizes_and_flags(built):
    import torch
    _, f = _fn()
    rng = np.random.default_rng(7)
    for n, b in ((1, 1), (255, 2), (256, 3), (257, 3), (100003, 3)):
        r = rng.standard_normal(n * b) * 10.0 ** rng.integers(-6, 6, n * b)
        skip = (rng.random(n) < 0.1).astype(np.int32)
        keep = np.repeat(skip == 0, b)
        want = float(np.abs(r[keep]).max()) if keep.any() else 0.0
        d_r, d_s = _device(r), _device(skip)
        torch.cuda.synchronize()
        for _ in range(2):
            st, err = _call(f, d_r.data_ptr(), d_s.data_ptr(), n, b)
            assert st == 0 and err == want, (n, b, err, want)
    # every cell skipped and no cells at all: error 0
    d_r = _device(np.ones(6))
    d_s = _device(np.ones(2, np.int32))
    torch.cuda.synchronize()
    assert _call(f, d_r.data_ptr(), d_s.data_ptr(), 2, 3) == (0, 0.0)
    assert _call(f, d_r.data_ptr(), None, 0, 3) == (0, 0.0)


def test_noalloc_nonfinite_and_limits(built):
    import torch
    lib, f = _fn()
    r = np.ones(3000)
    r[1234] = np.nan
    d_r = _device(r)
    torch.cuda.synchronize()
    st, err = _call(f, d_r.data_ptr(), None, 1000, 3)
    assert st == capi.ERR_NONFINITE and np.isnan(err)
    # the non-finite entry in a skipped cell does not count
    skip = np.zeros(1000, np.int32)
    skip[1234 // 3] = 1
    d_s = _device(skip)
    torch.cuda.synchronize()
    assert _call(f, d_r.data_ptr(), d_s.data_ptr(), 1000, 3) == (0, 1.0)
    # beyond the scratch limit: rejected on the host before any launch
    st, _ = _call(f, d_r.data_ptr(), None, MAX_CELLS + 1, 3)
    assert st == capi.ERR_ARG
    assert b"GBFV_NOALLOC_MAX_CELLS" in lib.gbfv_last_error()


def test_noalloc_allocates_no_device_memory(built):
    import torch
    _, f = _fn()
    d_r = _device(np.arange(3 * 50000, dtype=float))
    torch.cuda.synchronize()
    assert _call(f, d_r.data_ptr(), None, 50000, 3) == (0, 3 * 50000 - 1.0)  # set-up call
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(f, d_r.data_ptr(), None, 50000, 3) == (0, 3 * 50000 - 1.0)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
