"""Python view of libgbfv (the C ABI in include/gbfv.h).

The product is the CUDA library; this module only marshals numpy arrays
through ctypes.  Class and method names follow the reference interfaces the
entry points replace (FvBaseLinearizer, the linear-solver backend,
NewtonMethod).  There is no CPU fallback: constructing a Context without the
built library or without a GPU raises.
"""
import ctypes as C

import numpy as np

from . import capi, problems  # noqa: F401

__all__ = ["Context", "LinearSolver", "Batch", "capi", "problems", "default_params"]

default_params = capi.default_params


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Context:
    """One grid on the GPU: linearizer + BiCGStab/ILU0 backend + Newton."""

    def __init__(self, problem, params=None, set_initial=True, handle=None):
        self.lib = capi.load()
        self.problem = problem
        self.params = params if params is not None else capi.default_params()
        self._owned = handle is None
        if handle is None:
            self._s = problem.struct()
            st = C.c_int()
            self.h = self.lib.gbfv_create(C.byref(self._s), C.byref(self.params), C.byref(st))
            if not self.h:
                capi.check(st.value, "gbfv_create")
        else:
            self.h = handle
        n, b, nnz = C.c_int(), C.c_int(), C.c_int()
        self.lib.gbfv_dims(self.h, C.byref(n), C.byref(b), C.byref(nnz))
        self.N, self.b, self.nnz = n.value, b.value, nnz.value
        if set_initial and problem.init_pv is not None:
            self.set_solution(problem.init_pv, problem.init_meaning)

    def close(self):
        if getattr(self, "h", None):
            if self._owned:
                self.lib.gbfv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self.params = params
        capi.check(self.lib.gbfv_set_params(self.h, C.byref(params)), "gbfv_set_params")

    # model().solution(0)
    def set_solution(self, pv, meaning=None):
        pv = np.ascontiguousarray(pv, float)
        m = None if meaning is None else np.ascontiguousarray(meaning, np.int32)
        capi.check(self.lib.gbfv_set_solution(self.h, _d(pv), _i(m) if m is not None else None),
                   "gbfv_set_solution")

    def solution(self):
        pv = np.zeros(self.N * self.b)
        m = np.zeros(self.N, np.int32)
        capi.check(self.lib.gbfv_get_solution(self.h, _d(pv), _i(m)), "gbfv_get_solution")
        return pv, m

    # Simulator::serialize / deserialize (restart files, gbfv.restart)
    def write_restart(self, path, info):
        capi.check(self.lib.gbfv_write_restart(self.h, path.encode(), C.byref(info)), "gbfv_write_restart")

    def read_restart(self, path, info):
        """Read the solution from a restart file; returns its Simulator section."""
        out = capi.RestartInfo.from_buffer_copy(info)
        capi.check(self.lib.gbfv_read_restart(self.h, path.encode(), C.byref(out)), "gbfv_read_restart")
        return out

    # FvBaseLinearizer
    def linearize(self, dt, newton_iter=0):
        self.lib.gbfv_set_timestep(self.h, dt)
        self.lib.gbfv_set_newton_iteration(self.h, newton_iter)
        return self.lib.gbfv_linearize(self.h)

    def residual(self):
        r = np.zeros(self.N * self.b)
        capi.check(self.lib.gbfv_get_residual(self.h, _d(r)), "gbfv_get_residual")
        return r

    def jacobian(self):
        rp = np.zeros(self.N + 1, np.int32)
        col = np.zeros(self.nnz, np.int32)
        blk = np.zeros(self.nnz * self.b * self.b)
        capi.check(self.lib.gbfv_get_jacobian(self.h, _i(rp), _i(col), _d(blk)), "gbfv_get_jacobian")
        return rp, col, blk.reshape(self.nnz, self.b, self.b)

    def newton_error(self):
        e = C.c_double()
        st = self.lib.gbfv_newton_error(self.h, C.byref(e))
        return st, e.value

    # linear-solver backend
    def solve(self, want_dx=True):
        dx = np.zeros(self.N * self.b) if want_dx else None
        it = C.c_int()
        st = self.lib.gbfv_solve(self.h, _d(dx) if want_dx else None, C.byref(it))
        return st, dx, it.value

    # NewtonMethod
    def newton_update(self):
        sw = C.c_int()
        st = self.lib.gbfv_newton_update(self.h, C.byref(sw))
        return st, sw.value

    def newton_apply(self, dt):
        rep = capi.NewtonReport()
        st = self.lib.gbfv_newton_apply(self.h, dt, C.byref(rep))
        return st, rep

    def time_integration(self, steps, dt0, end_time=1e100, fixed_dt=False):
        sdt = np.zeros(steps)
        sn = np.zeros(steps, np.int32)
        sl = np.zeros(steps, np.int32)
        tl = C.c_int32()
        st = self.lib.gbfv_time_integration(self.h, steps, dt0, end_time, int(fixed_dt),
                                            _d(sdt), _i(sn), _i(sl), C.byref(tl))
        return st, sdt, sn, sl, tl.value

    def stream(self):
        return self.lib.gbfv_stream(self.h)

    def amg_levels(self):
        """Rows and colours of every level of the context's AMG hierarchy
        (empty before its first AMG solve)."""
        sizes = np.zeros(15, np.int32)
        colors = np.zeros(15, np.int32)
        n = self.lib.gbfv_amg_levels(self.h, _i(sizes), _i(colors))
        if n < 0:
            capi.check(-n, "gbfv_amg_levels")
        return sizes[:n], colors[:n]

    def save_state(self):
        capi.check(self.lib.gbfv_save_state(self.h), "gbfv_save_state")

    def restore_state(self):
        capi.check(self.lib.gbfv_restore_state(self.h), "gbfv_restore_state")

    def kernel_stats(self):
        k = capi.KernelStats()
        capi.check(self.lib.gbfv_get_kernel_stats(self.h, C.byref(k)), "gbfv_get_kernel_stats")
        return {f: getattr(k, f) for f, _ in capi.KernelStats._fields_}

    def solver_config(self, precision):
        mode, nb, nt = C.c_int(), C.c_int(), C.c_int()
        ms = np.zeros(16)
        self.lib.gbfv_solver_config(self.h, precision, C.byref(mode), C.byref(nb), _d(ms), C.byref(nt))
        if mode.value & capi.SOLVER_GILU:
            name = "gilu+tagged" if mode.value & capi.SOLVER_TAGGED else "gilu"
            return {"mode": name, "blocks": nb.value, "tune_ms": []}
        name = {0: "grid", 1: "cluster", 2: "hybrid"}.get(mode.value & 3, "?")
        if mode.value & capi.SOLVER_NARROW:
            name += "-256"
        if mode.value & capi.SOLVER_TILES:
            name += "+tiles"
        return {"mode": name, "blocks": nb.value,
                "tune_ms": ms[:nt.value].tolist()}

    def set_solver_config(self, precision, mode, blocks):
        """Fix the persistent solver's launch configuration (mode 0 = grid,
        1 = cluster, 2 = hybrid; or-ed with capi.SOLVER_TILES: spatial-tile
        sweeps)."""
        capi.check(self.lib.gbfv_set_solver_config(self.h, precision, mode, blocks), "gbfv_set_solver_config")

    def reset_kernel_stats(self):
        self.lib.gbfv_reset_kernel_stats(self.h)

    def phase_times(self):
        a = np.zeros(4)
        self.lib.gbfv_phase_times(self.h, _d(a))
        return a


class LinearSolver:
    """Stand-alone BiCGStab backend over a host BCRS matrix: block ILU(0)
    (ParallelBiCGStabSolverBackend) or, with params.linear_solver =
    LINSOLVER_AMG, the aggregation AMG V-cycle (ParallelAmgBackend)."""

    def __init__(self, row_ptr, col, b, params=None):
        self.lib = capi.load()
        self.params = params if params is not None else capi.default_params()
        self.rp = np.ascontiguousarray(row_ptr, np.int32)
        self.col = np.ascontiguousarray(col, np.int32)
        self.n = len(self.rp) - 1
        self.b = b
        st = C.c_int()
        self.h = self.lib.gbfv_linsolver_create(self.n, b, _i(self.rp), _i(self.col),
                                                C.byref(self.params), C.byref(st))
        if not self.h:
            capi.check(st.value, "gbfv_linsolver_create")

    def set_matrix(self, blocks):
        blocks = np.ascontiguousarray(blocks, float)
        capi.check(self.lib.gbfv_linsolver_set_matrix(self.h, _d(blocks)), "set_matrix")

    def solve(self, rhs):
        rhs = np.ascontiguousarray(rhs, float)
        x = np.zeros(self.n * self.b)
        it = C.c_int()
        st = self.lib.gbfv_linsolver_solve(self.h, _d(rhs), _d(x), C.byref(it))
        return st, x, it.value

    def amg_levels(self):
        """Rows and colours of every level of the AMG hierarchy (built from
        the matrix last set)."""
        sizes = np.zeros(15, np.int32)
        colors = np.zeros(15, np.int32)
        n = self.lib.gbfv_linsolver_amg_levels(self.h, _i(sizes), _i(colors))
        if n < 0:
            capi.check(-n, "gbfv_linsolver_amg_levels")
        return sizes[:n], colors[:n]

    def amg_apply(self, d):
        """One FP64 V-cycle v = M^-1 d of the AMG preconditioner."""
        d = np.ascontiguousarray(d, float)
        v = np.zeros(self.n * self.b)
        capi.check(self.lib.gbfv_linsolver_amg_apply(self.h, _d(d), _d(v)), "gbfv_linsolver_amg_apply")
        return v

    def ilu0_apply(self, d):
        """One FP64 application v = (LU)^-1 d of the general block ILU(0)
        (patterns beyond the 5/7-point stencil's)."""
        d = np.ascontiguousarray(d, float)
        v = np.zeros(self.n * self.b)
        capi.check(self.lib.gbfv_linsolver_ilu0_apply(self.h, _d(d), _d(v)), "gbfv_linsolver_ilu0_apply")
        return v

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbfv_linsolver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent systems advanced together (gbfv_batch_*): one batched
    launch per phase for all of them, each phase a replayed CUDA graph, one
    persistent BiCGStab/ILU0 launch whose clusters take systems from a queue."""

    def __init__(self, problems, params=None, cluster_size=0, set_initial=True):
        self.lib = capi.load()
        self.problems = list(problems)
        self.params = params if params is not None else capi.default_params()
        self._structs = [p.struct() for p in self.problems]
        arr = (capi.Problem * len(self._structs))(*self._structs)
        st = C.c_int()
        self.h = self.lib.gbfv_batch_create(arr, len(self._structs), C.byref(self.params), cluster_size,
                                            C.byref(st))
        if not self.h:
            capi.check(st.value, "gbfv_batch_create")
        self.systems = [Context(p, self.params, set_initial=False, handle=self.lib.gbfv_batch_system(self.h, i))
                        for i, p in enumerate(self.problems)]
        if set_initial:
            for c, p in zip(self.systems, self.problems):
                if p.init_pv is not None:
                    c.set_solution(p.init_pv, p.init_meaning)

    def __len__(self):
        return len(self.systems)

    def time_integration(self, steps, dt0, end_time=1e100, fixed_dt=False):
        return self.lib.gbfv_batch_time_integration(self.h, steps, dt0, end_time, int(fixed_dt))

    def autotune(self, dt):
        """Pick the cluster size of the batched solve by timing each candidate."""
        c, n = C.c_int(), C.c_int()
        ms = np.zeros(8)
        capi.check(self.lib.gbfv_batch_autotune(self.h, dt, C.byref(c), _d(ms), C.byref(n)), "gbfv_batch_autotune")
        return c.value, ms[:n.value].copy()

    def report(self, i):
        """Status, per-step dt / Newton / linear iterations and the number of
        linearizations of system i's last time integration."""
        st, n, nl = C.c_int(), C.c_int(), C.c_int()
        # the step count first, then arrays of exactly that many entries
        capi.check(self.lib.gbfv_batch_system_report(self.h, i, None, C.byref(n), None, None, None, None),
                   "gbfv_batch_system_report")
        k = n.value
        sdt = np.zeros(max(k, 1))
        sn = np.zeros(max(k, 1), np.int32)
        sl = np.zeros(max(k, 1), np.int32)
        capi.check(self.lib.gbfv_batch_system_report(self.h, i, C.byref(st), C.byref(n), _d(sdt), _i(sn), _i(sl),
                                                     C.byref(nl)), "gbfv_batch_system_report")
        return st.value, sdt[:k].copy(), sn[:k].copy(), sl[:k].copy(), nl.value

    def stats(self):
        s = capi.BatchStats()
        capi.check(self.lib.gbfv_batch_get_stats(self.h, C.byref(s)), "gbfv_batch_get_stats")
        return {f: getattr(s, f) for f, _ in capi.BatchStats._fields_}

    def stream(self):
        return self.lib.gbfv_batch_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            for c in self.systems:
                c.h = None
            self.lib.gbfv_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
