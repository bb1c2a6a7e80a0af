"""ctypes mirrors of the C structs declared in include/gbfv.h, and the loader
of the in-tree CUDA library.

The library is never pip-installed: it is built in-tree by
``__graft_entry__.build()`` into ``opm-models_gb300/_build/libgbfv.so``.  If it
is missing, :func:`load` raises -- there is no CPU fallback.
"""
import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libgbfv.so")

# status codes (enum gbfv_status)
OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_OOM = 3
ERR_NUMERICAL = 4
ERR_NONFINITE = 5
ERR_BREAKDOWN = 6
ERR_NOT_CONVERGED = 7
ERR_TIMEOUT = 8
ERR_UNSUPPORTED = 9
ERR_SINGULAR = 10
ERR_NO_DEVICE = 11
STATUS_NAMES = {
    0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_OOM", 4: "ERR_NUMERICAL",
    5: "ERR_NONFINITE", 6: "ERR_BREAKDOWN", 7: "ERR_NOT_CONVERGED",
    8: "ERR_TIMEOUT", 9: "ERR_UNSUPPORTED", 10: "ERR_SINGULAR", 11: "ERR_NO_DEVICE",
}

MODEL_IMMISCIBLE_2P = 0
MODEL_BLACKOIL_3P = 1
LAW_REG_VAN_GENUCHTEN = 0
LAW_REG_BROOKS_COREY = 1
LAW_COREY3P = 2
BC_NOFLOW = 0
BC_FREEFLOW = 1
BC_MASSRATE = 2
GAS_SG = 0
GAS_RS = 1
GAS_RV = 2
PREC_FP64 = 0
PREC_MIXED = 1

# persistent solver launch modes (gbfv_set_solver_config)
SOLVER_GRID = 0
SOLVER_CLUSTER = 1
SOLVER_HYBRID = 2
SOLVER_TILES = 4   # or-ed into SOLVER_CLUSTER / SOLVER_HYBRID: spatial-tile sweeps
SOLVER_NARROW = 8  # or-ed into SOLVER_HYBRID (mixed precision): 256-thread blocks
SOLVER_GILU = 16   # reported: the general block ILU(0) kernel
SOLVER_TAGGED = 32  # reported with SOLVER_GILU: tagged sweeps, no barrier per level
LIN_AD = 0         # local linearizer: automatic differentiation
LIN_FD = 1         # finite differences (FvBaseFdLocalLinearizer)
LINSOLVER_ILU0 = 0  # linear solver: BiCGStab + block ILU(0)
LINSOLVER_AMG = 1   # BiCGStab + aggregation AMG V-cycle (ParallelAmgBackend)
LINEARIZER_ELEMENT = 0  # FvBaseLinearizer (rows divided by the cell volume)
LINEARIZER_TPFA = 1     # TpfaLinearizer + BlackOilLocalResidualTPFA
MAX_CELLS = 33554368  # GBFV_MAX_CELLS: largest grid / block-row count (32-bit device indexing)
FLUX_DARCY = 0
FLUX_TRANS = 1
MAT_STRIDE = 8

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int32)


class BlackOilPvt(C.Structure):
    _fields_ = [
        ("rho_ref_oil", C.c_double), ("rho_ref_water", C.c_double), ("rho_ref_gas", C.c_double),
        ("n_oil", C.c_int32), ("oil_p", dp), ("oil_rs", dp), ("oil_bo", dp), ("oil_mu", dp),
        ("oil_compressibility", C.c_double),
        ("n_gas", C.c_int32), ("gas_p", dp), ("gas_bg", dp), ("gas_mu", dp),
        ("water_p_ref", C.c_double), ("water_bw_ref", C.c_double),
        ("water_compressibility", C.c_double), ("water_mu", C.c_double),
    ]


class Problem(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("num_cells", C.c_int32), ("num_conn", C.c_int32),
        ("num_bfaces", C.c_int32),
        ("center", dp), ("volume", dp), ("porosity", dp), ("perm", dp), ("material", ip),
        ("conn_ptr", ip), ("conn_nbr", ip), ("conn_dir", ip), ("conn_normal", dp),
        ("conn_center", dp), ("conn_area", dp),
        ("bface_ptr", ip), ("bface_normal", dp), ("bface_center", dp), ("bface_area", dp),
        ("bface_type", ip), ("bface_value", dp),
        ("constraint", ip), ("num_constraints", C.c_int32), ("constraint_pv", dp),
        ("constraint_meaning", ip),
        ("gravity", C.c_double * 3), ("num_materials", C.c_int32), ("material_params", dp),
        ("rho", C.c_double * 2), ("mu", C.c_double * 2),
        ("pvt", C.POINTER(BlackOilPvt)), ("temperature", C.c_double),
        ("flux_module", C.c_int32),
        ("num_elements", C.c_int32), ("elem_corner", ip), ("bface_corner", ip),
        ("p1_gradients", C.c_int32),
    ]


class Params(C.Structure):
    _fields_ = [
        ("newton_tolerance", C.c_double), ("newton_max_iterations", C.c_int32),
        ("newton_target_iterations", C.c_int32), ("newton_max_error", C.c_double),
        ("linear_tolerance", C.c_double), ("linear_abs_tolerance", C.c_double),
        ("linear_max_iterations", C.c_int32), ("linear_max_error", C.c_double),
        ("precision", C.c_int32), ("inner_tolerance", C.c_double),
        ("max_refinements", C.c_int32), ("dp_max_rel", C.c_double), ("ds_max", C.c_double),
        ("pv_oscillation_threshold", C.c_double), ("pressure_min", C.c_double),
        ("pressure_max", C.c_double), ("max_water_saturation", C.c_double),
        ("water_only_threshold", C.c_double), ("min_time_step", C.c_double),
        ("max_time_step", C.c_double), ("max_time_step_divisions", C.c_int32),
        ("local_linearizer", C.c_int32), ("numeric_difference_method", C.c_int32),
        ("linear_solver", C.c_int32), ("amg_coarsen_target", C.c_int32),
        ("linearizer", C.c_int32),
    ]


class KernelStats(C.Structure):
    _fields_ = [
        ("solve_ms", C.c_double), ("solve_launches", C.c_int64), ("solve_iterations", C.c_int64),
        ("solve_factorizations", C.c_int64), ("solve_bytes", C.c_double),
        ("linearize_ms", C.c_double), ("linearize_launches", C.c_int64),
        ("linearize_bytes", C.c_double),
    ]


class NewtonReport(C.Structure):
    _fields_ = [
        ("converged", C.c_int32), ("iterations", C.c_int32), ("linear_iterations", C.c_int32),
        ("linearizations", C.c_int32), ("refinements", C.c_int32), ("status", C.c_int32),
        ("error", C.c_double),
    ]


def default_params(**overrides):
    """The reference's parameter defaults (newtonmethodparameters.hh:31-53,
    linalgparameters.hh:41-78, blackoilnewtonmethodparameters.hh)."""
    p = Params()
    p.newton_tolerance = 1e-8
    p.newton_max_iterations = 20
    p.newton_target_iterations = 10
    p.newton_max_error = 1e100
    p.linear_tolerance = 1e-3
    p.linear_abs_tolerance = -1.0
    p.linear_max_iterations = 1000
    p.linear_max_error = 1e7
    p.precision = PREC_FP64
    p.inner_tolerance = 1e-3
    p.max_refinements = 20
    p.dp_max_rel = 0.3
    p.ds_max = 0.2
    p.pv_oscillation_threshold = 1e-5
    p.pressure_min = -1e99
    p.pressure_max = 1e99
    p.max_water_saturation = 1.0
    p.water_only_threshold = 1.0
    p.min_time_step = 0.0
    p.max_time_step = float("inf")
    p.max_time_step_divisions = 10
    p.local_linearizer = LIN_AD
    p.numeric_difference_method = 1
    p.linear_solver = LINSOLVER_ILU0
    p.amg_coarsen_target = 5000     # AmgCoarsenTarget (parallelamgbackend.hh:72)
    p.linearizer = LINEARIZER_ELEMENT
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def as_ptr(a, ctype):
    """Pointer to a contiguous numpy array (the array must stay alive)."""
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


class BatchStats(C.Structure):
    _fields_ = [("num_systems", C.c_int32), ("cluster_size", C.c_int32), ("num_clusters", C.c_int32),
                ("pad", C.c_int32), ("rounds", C.c_int64), ("graph_launches", C.c_int64),
                ("kernel_launches", C.c_int64), ("solve_launches", C.c_int64), ("solve_ms", C.c_double),
                ("solve_bytes", C.c_double), ("linearize_ms", C.c_double)]


class RestartInfo(C.Structure):
    """gbfv_restart_info: the restart file's cookie counts and Simulator section."""
    _fields_ = [("num_cpus", C.c_int32), ("rank", C.c_int32), ("num_edges", C.c_int32),
                ("num_vertices", C.c_int32), ("episode_index", C.c_int32), ("time_step_index", C.c_int32),
                ("episode_start_time", C.c_double), ("episode_length", C.c_double),
                ("start_time", C.c_double), ("time", C.c_double), ("vtk_section", C.c_int32),
                ("vtk_writer_num", C.c_int32), ("entity_codim", C.c_int32), ("num_elements", C.c_int32)]


_LIB = None


def load():
    """Load the in-tree CUDA library; raise if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libgbfv.so is not built (%s); run __graft_entry__.build() -- there is "
            "no CPU fallback" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    sig = {
        "gbfv_default_params": (None, [C.POINTER(Params)]),
        "gbfv_create": (vp, [C.POINTER(Problem), C.POINTER(Params), C.POINTER(C.c_int)]),
        "gbfv_destroy": (C.c_int, [vp]),
        "gbfv_set_params": (C.c_int, [vp, C.POINTER(Params)]),
        "gbfv_dims": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "gbfv_set_solution": (C.c_int, [vp, dp, ip]),
        "gbfv_get_solution": (C.c_int, [vp, dp, ip]),
        "gbfv_set_timestep": (C.c_int, [vp, C.c_double]),
        "gbfv_set_newton_iteration": (C.c_int, [vp, C.c_int]),
        "gbfv_linearize": (C.c_int, [vp]),
        "gbfv_get_residual": (C.c_int, [vp, dp]),
        "gbfv_get_jacobian": (C.c_int, [vp, ip, ip, dp]),
        "gbfv_newton_error": (C.c_int, [vp, dp]),
        "gbfv_solve": (C.c_int, [vp, dp, C.POINTER(C.c_int)]),
        "gbfv_newton_update": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "gbfv_newton_apply": (C.c_int, [vp, C.c_double, C.POINTER(NewtonReport)]),
        "gbfv_suggest_time_step": (C.c_double, [vp, C.c_double, C.c_int]),
        "gbfv_time_integration": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int,
                                            dp, ip, ip, ip]),
        "gbfv_linsolver_create": (vp, [C.c_int, C.c_int, ip, ip, C.POINTER(Params),
                                       C.POINTER(C.c_int)]),
        "gbfv_linsolver_destroy": (C.c_int, [vp]),
        "gbfv_linsolver_set_matrix": (C.c_int, [vp, dp]),
        "gbfv_linsolver_solve": (C.c_int, [vp, dp, dp, C.POINTER(C.c_int)]),
        "gbfv_linsolver_amg_levels": (C.c_int, [vp, ip, ip]),
        "gbfv_amg_levels": (C.c_int, [vp, ip, ip]),
        "gbfv_linsolver_amg_apply": (C.c_int, [vp, dp, dp]),
        "gbfv_linsolver_ilu0_apply": (C.c_int, [vp, dp, dp]),
        "gbfv_kernel_launches": (C.c_int64, []),
        "gbfv_last_error": (C.c_char_p, []),
        "gbfv_phase_times": (C.c_int, [vp, dp]),
        "gbfv_stream": (vp, [vp]),
        "gbfv_save_state": (C.c_int, [vp]),
        "gbfv_restore_state": (C.c_int, [vp]),
        "gbfv_get_kernel_stats": (C.c_int, [vp, C.POINTER(KernelStats)]),
        "gbfv_reset_kernel_stats": (C.c_int, [vp]),
        "gbfv_solver_phase_ns": (C.c_int, [vp, C.POINTER(C.c_uint64)]),
        "gbfv_solver_config": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), dp,
                                         C.POINTER(C.c_int)]),
        "gbfv_set_solver_config": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
        "gbfv_batch_create": (vp, [C.POINTER(Problem), C.c_int, C.POINTER(Params), C.c_int,
                                   C.POINTER(C.c_int)]),
        "gbfv_batch_destroy": (C.c_int, [vp]),
        "gbfv_batch_system": (vp, [vp, C.c_int]),
        "gbfv_batch_time_integration": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int]),
        "gbfv_batch_system_report": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), dp, ip, ip,
                                               C.POINTER(C.c_int)]),
        "gbfv_batch_get_stats": (C.c_int, [vp, C.POINTER(BatchStats)]),
        "gbfv_batch_stream": (vp, [vp]),
        "gbfv_batch_autotune": (C.c_int, [vp, C.c_double, C.POINTER(C.c_int), dp, C.POINTER(C.c_int)]),
        "gbfv_footprint_bytes": (C.c_int64, [C.c_int, C.c_int, C.c_int]),
        "gbfv_serve_create": (vp, [C.c_int, C.c_int, C.POINTER(Params), C.c_int, C.c_int, C.POINTER(C.c_int)]),
        "gbfv_serve_admit": (C.c_int, [vp, C.POINTER(Problem), dp, ip, C.c_int, C.c_double, C.c_int,
                                       C.POINTER(C.c_int)]),
        "gbfv_serve_step": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "gbfv_serve_slot": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "gbfv_serve_release": (C.c_int, [vp, C.c_int]),
        "gbfv_serve_footprint": (C.c_int64, [vp]),
        "gbfv_selftest_wait_timeout": (C.c_int, [dp]),
        "gbfv_output_fields": (C.c_int, [vp, dp]),
        "gbfv_write_vtk": (C.c_int, [vp, vp, C.c_int32, C.c_char_p]),
        "gbfv_vtk_file_name": (C.c_int, [C.c_char_p, C.c_int32, C.c_char_p, C.c_size_t]),
        "gbfv_write_pvd": (C.c_int, [C.c_char_p, C.c_int32, dp, C.POINTER(C.c_char_p)]),
        "gbfv_format_restart": (C.c_int, [C.POINTER(RestartInfo), C.c_int32, C.c_int32, dp, ip, C.c_char_p,
                                          C.c_size_t, C.POINTER(C.c_size_t)]),
        "gbfv_parse_restart": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(RestartInfo), C.c_int32, C.c_int32,
                                         dp, ip, C.POINTER(RestartInfo)]),
        "gbfv_restart_file_name": (C.c_int, [C.c_char_p, C.c_char_p, C.c_double, C.c_int32, C.c_char_p,
                                             C.c_size_t]),
        "gbfv_write_restart": (C.c_int, [vp, C.c_char_p, C.POINTER(RestartInfo)]),
        "gbfv_read_restart": (C.c_int, [vp, C.c_char_p, C.POINTER(RestartInfo)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def exported_symbols():
    """Names of the entry points declared in include/gbfv.h."""
    hdr = os.path.join(os.path.dirname(PKG_ROOT), "include", "gbfv.h")
    import re
    names = []
    with open(hdr) as f:
        txt = f.read()
    for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(gbfv_\w+)\s*\(", txt, re.M):
        names.append(m.group(1))
    return sorted(set(names))


def check(status, what="gbfv call"):
    if status != OK:
        lib = load()
        msg = lib.gbfv_last_error().decode() if lib else ""
        raise RuntimeError("%s failed: %s %s" % (what, STATUS_NAMES.get(status, status), msg))


__all__ = [n for n in dir() if not n.startswith("_")] + ["np"]
