"""ctypes binding of the C ABI in include/phrike_gb300.h.

Field data crosses the boundary as raw device pointers (``tensor.data_ptr()``)
and the stream as ``torch.cuda.current_stream().cuda_stream``.  A non-zero
status becomes a RuntimeError carrying ``ps_last_error()``.  There is no
fallback: if the library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphrike_gb300.so")

PS_OK = 0
PS_BASIS_FOURIER = 0
PS_BASIS_LEGENDRE = 1
PS_EQ_EULER = 0
PS_EQ_MHD = 1
PS_AV_OFF, PS_AV_SENSOR, PS_AV_CONSTANT = 0, 1, 2
PS_TRACERS_AUTO, PS_TRACERS_EXACT, PS_TRACERS_NUFFT = 0, 1, 2
PS_AV_Q_DENSITY, PS_AV_Q_PRESSURE, PS_AV_Q_SPEED = 0, 1, 2
PS_OP_P, PS_OP_D, PS_OP_L = 0, 1, 2
PS_SCHEME_RK4, PS_SCHEME_RK2 = 0, 1
PS_GEMM_FP32 = 0
PS_GEMM_FP64 = 1
PS_GEMM_BF16X3 = 2
PS_GEMM_BF16X3_SIMT = 3
GEMM_PRECISIONS = {"fp32": PS_GEMM_FP32, "fp64": PS_GEMM_FP64, "bf16x3": PS_GEMM_BF16X3,
                   "bf16x3_simt": PS_GEMM_BF16X3_SIMT}
KIND_NAMES = ["x_pass", "y_pass", "last_pass", "op_pass", "step1d", "lgl_x", "lgl_y"]


class PlanDesc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int),
        ("n", C.c_int * 3),
        ("length", C.c_double * 3),
        ("basis", C.c_int * 3),
        ("equations", C.c_int),
        ("gamma", C.c_double),
        ("dealias", C.c_int),
        ("filter_enabled", C.c_int),
        ("filter_p", C.c_int),
        ("filter_alpha", C.c_double),
        ("filter_interval", C.c_int),
        ("gravity", C.c_double * 3),
        ("cfl", C.c_double),
        ("gemm_precision", C.c_int),
        ("mhd_rho_min", C.c_double),
        ("mhd_p_min", C.c_double),
        ("mhd_project_substages", C.c_int),
        ("mhd_divergence_clean", C.c_int),
        ("mhd_resistivity", C.c_double),
        ("mhd_viscosity", C.c_double),
        ("av_mode", C.c_int),
        ("av_sensor", C.c_int),
        ("av_nu_max", C.c_double),
        ("av_nu_constant", C.c_double),
        ("av_s_ref", C.c_double),
        ("av_s_min", C.c_double),
        ("av_p", C.c_double),
        ("av_epsilon", C.c_double),
        ("av_weight", C.c_double * 5),
        ("scheme", C.c_int),
        ("mhd_cfl_diff", C.c_double),
        ("lgl_bc1d", C.c_int * 6),
        ("tile_cols", C.c_int),
        ("umma_n_tile", C.c_int),
    ]


PS_ARK_RK23, PS_ARK_RK45, PS_ARK_RK78 = 0, 1, 2
ARK_METHODS = {"rk23": PS_ARK_RK23, "rk45": PS_ARK_RK45, "rk78": PS_ARK_RK78}


class AdaptiveDesc(C.Structure):
    """ps_adaptive_desc (include/phrike_gb300.h)."""
    _fields_ = [
        ("method", C.c_int),
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("safety_factor", C.c_double),
        ("min_dt_factor", C.c_double),
        ("max_dt_factor", C.c_double),
        ("max_rejections", C.c_int),
    ]


# (name, restype, argtypes) of every exported entry point
_SIGNATURES = [
    ("ps_plan_desc_init", C.c_int, [C.POINTER(PlanDesc), C.c_int]),
    ("ps_plan_scratch_bytes", C.c_int, [C.POINTER(PlanDesc), C.POINTER(C.c_size_t)]),
    ("ps_plan_create", C.c_int, [C.POINTER(PlanDesc), C.POINTER(C.c_void_p)]),
    ("ps_plan_destroy", C.c_int, [C.c_void_p]),
    ("ps_batch_create", C.c_int, [C.POINTER(PlanDesc), C.c_int, C.POINTER(C.c_void_p)]),
    ("ps_batch_scratch_bytes", C.c_int, [C.POINTER(PlanDesc), C.c_int, C.POINTER(C.c_size_t)]),
    ("ps_plan_nsolve", C.c_int, [C.c_void_p]),
    ("ps_plan_steps_done", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("ps_run_cfl", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_adaptive_desc_init", None, [C.POINTER(AdaptiveDesc)]),
    ("ps_run_adaptive", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(AdaptiveDesc), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_adaptive_reset", C.c_int, [C.c_void_p, C.c_void_p]),
    ("ps_rhs", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_step_rk4", C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    ("ps_run_steps", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p]),
    ("ps_derivative", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("ps_filter", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("ps_max_wave_speed", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_conserved", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_plan_ncomp", C.c_int, [C.c_void_p]),
    ("ps_plan_tile_cols", C.c_int, [C.c_void_p]),
    ("ps_plan_status", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("ps_profile_enable", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_profile_collect", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]),
    ("ps_tracer_method", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_rhs_static", C.c_int, [C.POINTER(PlanDesc), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_lgl_build", C.c_int, [C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_apply_boundary_conditions", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_project_solenoidal", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_project_state", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_project_solenoidal_3d", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_axis_op", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("ps_eval_points", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    ("ps_tracers_step", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                  C.c_void_p, C.c_void_p]),
    ("ps_last_error", C.c_char_p, []),
    ("ps_version", C.c_char_p, []),
]

_lib = None
_lock = threading.Lock()


def exported_names():
    return [n for n, _, _ in _SIGNATURES]


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the shared library (build it first with phrike_gb300._build.build())."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} not found: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(path)
        for name, res, args in _SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != PS_OK:
        msg = load().ps_last_error().decode(errors="replace")
        raise RuntimeError(f"phrike_gb300 error {rc}: {msg}")
