"""ORACLE -- test infrastructure only.

ctypes binding of the CPU restatement (oracle/oracle.cc).  Only tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may
import this module; the product path never does.  Parity status: unpinned
against the reference's own output (the reference cannot be built here);
the oracle's table of unpinned choices lists what it restates.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# GBFV_ORACLE_LIB selects another build of the same source (the sanitizer
# build of the Makefile's `sanitize` target)
LIB = os.environ.get("GBFV_ORACLE_LIB") or os.path.join(HERE, "_build", "liboracle.so")


def build(quiet=True):
    """Compile the oracle with its Makefile (gcc/g++, OpenMP)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "opm-models_gb300"))
    from gbfv import capi  # struct layouts only
    lib = C.CDLL(LIB)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    sig = {
        "oracle_default_params": (None, [C.POINTER(capi.Params)]),
        "oracle_create": (vp, [C.POINTER(capi.Problem), C.POINTER(capi.Params)]),
        "oracle_destroy": (None, [vp]),
        "oracle_set_threads": (None, [C.c_int]),
        "oracle_get_threads": (C.c_int, []),
        "oracle_set_dot_lanes": (None, [C.c_int]),
        "oracle_output_fields": (C.c_int, [vp, dp]),
        "oracle_set_params": (C.c_int, [vp, C.POINTER(capi.Params)]),
        "oracle_set_solution": (C.c_int, [vp, dp, ip]),
        "oracle_get_solution": (C.c_int, [vp, dp, ip]),
        "oracle_nnz": (C.c_int, [vp]),
        "oracle_linearize": (C.c_int, [vp, C.c_double, C.c_int]),
        "oracle_get_residual": (C.c_int, [vp, dp]),
        "oracle_get_storage_old": (C.c_int, [vp, dp]),
        "oracle_get_residual_scale": (C.c_int, [vp, dp]),
        "oracle_get_jacobian": (C.c_int, [vp, ip, ip, dp]),
        "oracle_newton_error": (C.c_int, [vp, dp]),
        "oracle_solve": (C.c_int, [vp, dp, C.POINTER(C.c_int)]),
        "oracle_newton_update": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "oracle_newton_apply": (C.c_int, [vp, C.c_double, C.POINTER(capi.NewtonReport)]),
        "oracle_time_integration": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int,
                                              dp, ip, ip, ip]),
        "oracle_bcrs_solve": (C.c_int, [C.c_int, C.c_int, ip, ip, dp, dp, dp,
                                        C.POINTER(capi.Params), C.POINTER(C.c_int)]),
        "oracle_ilu0": (C.c_int, [C.c_int, C.c_int, ip, ip, dp, dp, dp, dp]),
        "oracle_amg": (C.c_int, [C.c_int, C.c_int, ip, ip, dp, C.c_int, ip, ip, ip, dp, dp]),
    }
    for n, (r, a) in sig.items():
        f = getattr(lib, n)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Oracle:
    """The reference algorithm on the CPU, same interface shape as gbfv.Context."""

    def __init__(self, problem, params):
        self.lib = load()
        self.problem = problem
        self.params = params
        self._s = problem.struct()
        self.h = self.lib.oracle_create(C.byref(self._s), C.byref(params))
        if not self.h:
            raise RuntimeError("oracle_create failed")
        self.N = problem.num_cells
        self.b = problem.b
        self.set_solution(problem.init_pv, problem.init_meaning)

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    __del__ = close

    def set_params(self, params):
        self.params = params
        self.lib.oracle_set_params(self.h, C.byref(params))

    def set_solution(self, pv, meaning=None):
        pv = np.ascontiguousarray(pv, float)
        m = None if meaning is None else np.ascontiguousarray(meaning, np.int32)
        self.lib.oracle_set_solution(self.h, _d(pv), _i(m) if m is not None else None)

    def solution(self):
        pv = np.zeros(self.N * self.b)
        m = np.zeros(self.N, np.int32)
        self.lib.oracle_get_solution(self.h, _d(pv), _i(m))
        return pv, m

    def linearize(self, dt, newton_iter=0):
        return self.lib.oracle_linearize(self.h, dt, newton_iter)

    def residual(self):
        r = np.zeros(self.N * self.b)
        self.lib.oracle_get_residual(self.h, _d(r))
        return r

    def output_fields(self):
        """[19, N]: the quantities the VTK output writes (layout of
        gbfv_output_fields)."""
        out = np.zeros(19 * self.N)
        self.lib.oracle_output_fields(self.h, _d(out))
        return out.reshape(19, self.N)

    def residual_scale(self):
        """Per-row sum of |terms| / V of the last linearization: the size of
        the quantities the residual sums, used as the parity scale."""
        r = np.zeros(self.N * self.b)
        self.lib.oracle_get_residual_scale(self.h, _d(r))
        return r

    def jacobian(self):
        nnz = self.lib.oracle_nnz(self.h)
        rp = np.zeros(self.N + 1, np.int32)
        col = np.zeros(nnz, np.int32)
        blk = np.zeros(nnz * self.b * self.b)
        self.lib.oracle_get_jacobian(self.h, _i(rp), _i(col), _d(blk))
        return rp, col, blk.reshape(nnz, self.b, self.b)

    def newton_error(self):
        e = C.c_double()
        self.lib.oracle_newton_error(self.h, C.byref(e))
        return e.value

    def solve(self):
        dx = np.zeros(self.N * self.b)
        it = C.c_int()
        st = self.lib.oracle_solve(self.h, _d(dx), C.byref(it))
        return st, dx, it.value

    def newton_update(self):
        sw = C.c_int()
        st = self.lib.oracle_newton_update(self.h, C.byref(sw))
        return st, sw.value

    def newton_apply(self, dt):
        from gbfv import capi
        rep = capi.NewtonReport()
        st = self.lib.oracle_newton_apply(self.h, dt, C.byref(rep))
        return st, rep

    def time_integration(self, steps, dt0, end_time=1e100, fixed_dt=False):
        sdt = np.zeros(steps)
        sn = np.zeros(steps, np.int32)
        sl = np.zeros(steps, np.int32)
        tl = C.c_int32()
        st = self.lib.oracle_time_integration(self.h, steps, dt0, end_time, int(fixed_dt),
                                              _d(sdt), _i(sn), _i(sl), C.byref(tl))
        return st, sdt, sn, sl, tl.value


def set_threads(n):
    load().oracle_set_threads(int(n))


def set_dot_lanes(lanes):
    """Summation order of the BiCGStab scalar products: 0 the reference's
    sequential sum, L > 0 L strided partial sums combined pairwise (another
    correct order, as a parallel machine sums)."""
    load().oracle_set_dot_lanes(int(lanes))


def bcrs_solve(rp, col, blocks, rhs, params):
    lib = load()
    n = len(rp) - 1
    b = blocks.shape[-1]
    x = np.zeros(n * b)
    it = C.c_int()
    rp = np.ascontiguousarray(rp, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    blocks = np.ascontiguousarray(blocks, float)
    rhs = np.ascontiguousarray(rhs, float)
    st = lib.oracle_bcrs_solve(n, b, _i(rp), _i(col), _d(blocks), _d(rhs), _d(x),
                               C.byref(params), C.byref(it))
    return st, x, it.value


def ilu0(rp, col, blocks, d=None):
    lib = load()
    n = len(rp) - 1
    b = blocks.shape[-1]
    rp = np.ascontiguousarray(rp, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    blocks = np.ascontiguousarray(blocks, float)
    F = np.zeros_like(blocks)
    v = np.zeros(n * b)
    dd = None if d is None else np.ascontiguousarray(d, float)
    st = lib.oracle_ilu0(n, b, _i(rp), _i(col), _d(blocks), _d(F),
                         _d(dd) if dd is not None else None, _d(v) if dd is not None else None)
    return st, F, v


def amg(rp, col, blocks, coarsen_target=5000, d=None):
    """The AMG hierarchy of a BCRS matrix (level sizes, level-0 aggregates and
    colours) and, with d, one V-cycle v = M^-1 d.  Returns (levels or a
    negative status, sizes, agg0, colors0, v)."""
    lib = load()
    n = len(rp) - 1
    b = blocks.shape[-1]
    rp = np.ascontiguousarray(rp, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    blocks = np.ascontiguousarray(blocks, float)
    sizes = np.zeros(15, np.int32)
    agg0 = np.zeros(n, np.int32)
    colors0 = np.zeros(n, np.int32)
    v = np.zeros(n * b)
    dd = None if d is None else np.ascontiguousarray(d, float)
    L = lib.oracle_amg(n, b, _i(rp), _i(col), _d(blocks), int(coarsen_target), _i(sizes), _i(agg0), _i(colors0),
                       _d(dd) if dd is not None else None, _d(v) if dd is not None else None)
    return L, sizes[:max(L, 0)], agg0, colors0, v
