"""ctypes binding of libgb300ocean.so (the C ABI declared in include/gbo.h).

The shared library is built in-tree by ``oceananigans_gb300.build.build()``.
Loading fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libgb300ocean.so")

GBO_OK = 0
GBO_ERR_INVALID = -1
GBO_ERR_CUDA = -2
GBO_ERR_NAN = -3
GBO_ERR_NOT_CONVERGED = -4
GBO_ERR_TIMEOUT = -5
GBO_ERR_NO_DEVICE = -6
GBO_ERR_STATE = -7

GBO_FLAT, GBO_PERIODIC, GBO_BOUNDED = 0, 1, 2
GBO_FLOAT32, GBO_FLOAT64 = 4, 8
GBO_ADVECTION_NONE, GBO_ADVECTION_CENTERED2, GBO_ADVECTION_WENO5 = 0, 2, 5
GBO_CLOSURE_NONE, GBO_CLOSURE_SMAGORINSKY_LILLY, GBO_CLOSURE_AMD, GBO_CLOSURE_SCALAR_DIFFUSIVITY = 0, 1, 2, 3
GBO_CLOSURE_DYNAMIC_SMAGORINSKY = 4
GBO_AVERAGING_XY, GBO_AVERAGING_LAGRANGIAN = 0, 1
GBO_TIMESTEPPER_RK3, GBO_TIMESTEPPER_QAB2 = 0, 1
GBO_SOLVER_FFT, GBO_SOLVER_FOURIER_TRIDIAGONAL, GBO_SOLVER_CONJUGATE_GRADIENT = 0, 1, 2
GBO_PRECOND_FFT, GBO_PRECOND_NONE, GBO_PRECOND_LEARNED = 0, 1, 2
GBO_FIELD_U, GBO_FIELD_V, GBO_FIELD_W, GBO_FIELD_TRACER = 0, 1, 2, 3
GBO_FIELD_PNHS, GBO_FIELD_PHY, GBO_FIELD_NU, GBO_FIELD_KAPPA = 100, 101, 102, 103
GBO_FIELD_JLM, GBO_FIELD_JMM = 104, 105
GBO_MAX_TRACERS = 4


class LaunchShape(ctypes.Structure):
    _fields_ = [("dct_columns", ctypes.c_int32), ("x_lines", ctypes.c_int32), ("y_columns", ctypes.c_int32),
                ("levels", ctypes.c_int32)]


class GridDesc(ctypes.Structure):
    _fields_ = [("size", ctypes.c_int32 * 3), ("topology", ctypes.c_int32 * 3),
                ("x", ctypes.c_double * 2), ("y", ctypes.c_double * 2), ("z", ctypes.c_double * 2),
                ("z_faces", ctypes.POINTER(ctypes.c_double)),
                ("bottom_height", ctypes.POINTER(ctypes.c_double)),
                ("float_type", ctypes.c_int32)]


class ModelDesc(ctypes.Structure):
    _fields_ = [("advection", ctypes.c_int32), ("closure", ctypes.c_int32),
                ("closure_C", ctypes.c_double), ("closure_Cb", ctypes.c_double), ("closure_Pr", ctypes.c_double),
                ("ntracers", ctypes.c_int32), ("buoyancy_tracer", ctypes.c_int32),
                ("has_coriolis", ctypes.c_int32), ("coriolis_f", ctypes.c_double),
                ("tracer_flux_top", ctypes.c_double * GBO_MAX_TRACERS),
                ("tracer_flux_bottom", ctypes.c_double * GBO_MAX_TRACERS),
                ("pressure_solver", ctypes.c_int32), ("preconditioner", ctypes.c_int32),
                ("cg_reltol", ctypes.c_double), ("cg_abstol", ctypes.c_double), ("cg_maxiter", ctypes.c_int32),
                ("closure_nu", ctypes.c_double), ("closure_kappa", ctypes.c_double * GBO_MAX_TRACERS),
                ("timestepper", ctypes.c_int32), ("ab2_chi", ctypes.c_double),
                ("closure_min_numerator", ctypes.c_double), ("closure_averaging", ctypes.c_int32)]


class GboError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class NotConvergedError(GboError):
    pass


class NaNError(GboError):
    pass


GBO_STOP_NONE, GBO_STOP_TIME, GBO_STOP_ITERATION, GBO_STOP_NAN, GBO_STOP_WALL_TIME = 0, 1, 2, 3, 4


class RunDesc(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("stop_time", ctypes.c_double), ("stop_iteration", ctypes.c_double),
                ("wall_time_limit", ctypes.c_double), ("align_time_step", ctypes.c_int32),
                ("minimum_relative_step", ctypes.c_double), ("nan_check_interval", ctypes.c_int32),
                ("nan_erroring", ctypes.c_int32), ("wizard_interval", ctypes.c_int32),
                ("cfl", ctypes.c_double), ("diffusive_cfl", ctypes.c_double),
                ("max_change", ctypes.c_double), ("min_change", ctypes.c_double),
                ("max_dt", ctypes.c_double), ("min_dt", ctypes.c_double),
                ("iterations_per_launch", ctypes.c_int32)]


class RunResult(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("time", ctypes.c_double), ("iteration", ctypes.c_int64),
                ("steps", ctypes.c_int64), ("stop_reason", ctypes.c_int32), ("nan_detected", ctypes.c_int32)]


# Every exported entry point with its ctypes signature.  The test suite checks
# that this table, include/gbo.h and the built library agree.
_vp = ctypes.c_void_p
SIGNATURES = {
    "gbo_model_desc_default": (None, [ctypes.POINTER(ModelDesc)]),
    "gbo_cg_parameters": (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(ModelDesc),
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "gbo_model_create": (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(ModelDesc), ctypes.POINTER(_vp)]),
    "gbo_model_destroy": (None, [_vp]),
    "gbo_set_field": (ctypes.c_int, [_vp, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int64]),
    "gbo_set_finalize": (ctypes.c_int, [_vp, ctypes.c_int32]),
    "gbo_get_field": (ctypes.c_int, [_vp, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int64]),
    "gbo_field_count": (ctypes.c_int64, [_vp, ctypes.c_int32]),
    "gbo_field_device_pointer": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.POINTER(_vp), ctypes.POINTER(ctypes.c_int64)]),
    "gbo_field_reference_profile": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.c_int64]),
    "gbo_time_step": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int32]),
    "gbo_clock": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
    "gbo_synchronize": (ctypes.c_int, [_vp]),
    "gbo_last_solver_iterations": (ctypes.c_int32, [_vp]),
    "gbo_last_error": (ctypes.c_char_p, [_vp]),
    "gbo_version": (ctypes.c_char_p, []),
    "gbo_poisson_solve_device": (ctypes.c_int, [_vp, _vp, _vp]),
    "gbo_learned_weight_count": (ctypes.c_int64, []),
    "gbo_learned_preconditioner": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int64]),
    "gbo_learned_trainer_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_float), ctypes.c_int64, ctypes.POINTER(_vp)]),
    "gbo_learned_trainer_destroy": (None, [_vp]),
    "gbo_learned_trainer_gradients": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_double),
                                                     ctypes.POINTER(ctypes.c_float)]),
    "gbo_learned_trainer_step": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_double,
                                                ctypes.POINTER(ctypes.c_double)]),
    "gbo_learned_trainer_weights": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "gbo_learned_trainer_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "gbo_poisson_operator_device": (ctypes.c_int, [_vp, _vp, _vp]),
    "gbo_precondition_device": (ctypes.c_int, [_vp, _vp, _vp]),
    "gbo_state_bytes": (ctypes.c_int64, [_vp]),
    "gbo_get_state": (ctypes.c_int, [_vp, _vp, ctypes.c_int64]),
    "gbo_set_state": (ctypes.c_int, [_vp, _vp, ctypes.c_int64]),
    "gbo_run_desc_default": (None, [ctypes.POINTER(RunDesc)]),
    "gbo_run": (ctypes.c_int, [_vp, ctypes.POINTER(RunDesc), ctypes.POINTER(RunResult)]),
    "gbo_cell_advection_timescale": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "gbo_cell_diffusion_timescale": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "gbo_ensemble_create": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(GridDesc), ctypes.POINTER(ModelDesc),
                                           ctypes.POINTER(_vp)]),
    "gbo_ensemble_destroy": (None, [_vp]),
    "gbo_ensemble_size": (ctypes.c_int32, [_vp]),
    "gbo_ensemble_member": (_vp, [_vp, ctypes.c_int32]),
    "gbo_ensemble_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "gbo_ensemble_time_step": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int32]),
    "gbo_poisson_solve_fft_static": (ctypes.c_int, [ctypes.POINTER(GridDesc), _vp, _vp, _vp]),
    "gbo_model_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "gbo_kernel_launches": (ctypes.c_int64, [_vp]),
    "gbo_kernel_timings": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.c_int32]),
    "gbo_kernel_group_count": (ctypes.c_int32, []),
    "gbo_kernel_timing_counts": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int32]),
    "gbo_kernel_group_name": (ctypes.c_char_p, [ctypes.c_int32]),
    "gbo_get_launch_shape": (ctypes.c_int, [_vp, ctypes.POINTER(LaunchShape)]),
    "gbo_set_launch_shape": (ctypes.c_int, [_vp, ctypes.POINTER(LaunchShape)]),
}

_lib = None


def load(path=None):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libgb300ocean.so not found at %s: run "
                           "`python -c 'import __graft_entry__ as g; g.build()'` first" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc, handle=None):
    if rc == GBO_OK:
        return
    L = load()
    msg = L.gbo_last_error(handle).decode(errors="replace")
    if rc == GBO_ERR_NOT_CONVERGED:
        raise NotConvergedError(rc, msg)
    if rc == GBO_ERR_NAN:
        raise NaNError(rc, msg)
    raise GboError(rc, msg)
