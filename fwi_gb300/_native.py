"""ctypes binding of libfwi_gb300.so (the C ABI in include/fwi_gb300.h).

The library is built in-tree (fwi_gb300/_lib).  Importing this module fails
loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfwi_gb300.so")

FWI_OK = 0
FWI_ERR_ARG = -1
FWI_ERR_CUDA = -2
FWI_ERR_NOMEM = -3
FWI_ERR_NONFINITE = -4
FWI_ERR_STATE = -5

SNAP_F32, SNAP_BF16, SNAP_F16 = 0, 1, 2
SURVEY_NO_GRAPH = 1
SURVEY_RECOMPUTE = 2
SURVEY_SINGLE_STEP = 4
SURVEY_FUSED_STEP = 8
SURVEY_GRAPH = 16
GRAD_F32, GRAD_F64 = 0, 1

EXPORTS = [
    "fwi_init", "fwi_finalize", "fwi_last_error", "fwi_set_stream", "fwi_set_solver_options",
    "fwi_kernel_launch_count", "fwi_solver_acoustic_ss", "fwi_misfit_function", "fwi_beta_calculous",
    "fwi_mcs_geometry", "fwi_ricker", "fwi_time_rules", "fwi_survey_create", "fwi_survey_destroy",
    "fwi_survey_set_lambda", "fwi_survey_set_observed", "fwi_survey_set_sources", "fwi_survey_run",
    "fwi_survey_grad_device", "fwi_survey_get_stack", "fwi_survey_get_synthetic", "fwi_survey_step_bytes", "fwi_survey_two_step_bytes", "fwi_survey_tuning",
    "fwi_survey_recompute", "fwi_survey_set_time", "fwi_time_filter", "fwi_set_filter_order",
    "fwi_interpolation_akima", "fwi_su_info", "fwi_su_read", "fwi_su_write", "fwi_read_nav",
    "fwi_survey_time_steps", "fwi_misfit_gradient_batch", "fwi_solver_forward_noalloc", "fwi_survey_tiles",
    "fwi_batch_plans", "fwi_batch_release", "fwi_first_step", "fwi_model_update", "fwi_was_geometry", "fwi_su_supershot", "fwi_survey_edge_tiles",
    "fwi_survey_launch_form", "fwi_survey_stepping", "fwi_batch_survey",
]


class FwiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fwi_gb300 error {code}: {msg}")
        self.code = code


class FwiShot(C.Structure):
    _fields_ = [("x0", C.c_int), ("nx", C.c_int), ("num_sou", C.c_int), ("num_rec", C.c_int),
                ("nxSou", C.c_void_p), ("nySou", C.c_void_p), ("nxRec", C.c_void_p), ("nyRec", C.c_void_p),
                ("src", C.c_void_p), ("obs", C.c_void_p), ("grad_weight", C.c_double), ("misfit_weight", C.c_double)]


class FwiSurveyDesc(C.Structure):
    _fields_ = [("ny", C.c_int), ("nx_model", C.c_int), ("d", C.c_float), ("dt", C.c_float), ("nt", C.c_int),
                ("store_snap", C.c_int), ("acc", C.c_int), ("dpml", C.c_int), ("numtasks", C.c_int),
                ("snap_form", C.c_int), ("grad_form", C.c_int), ("nshots", C.c_int),
                ("shots", C.POINTER(FwiShot)), ("water_rows", C.c_void_p), ("hbm_budget", C.c_size_t),
                ("wave_shots", C.c_int), ("band_rows", C.c_int), ("flags", C.c_int), ("tile_kernel", C.c_int),
                ("tile_rows", C.c_int), ("tile_edge_rows", C.c_int)]


_lib = None


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m fwi_gb300.build` "
                          "(the FWI path has no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    P, I, F, D = C.c_void_p, C.c_int, C.c_float, C.c_double
    IP = C.POINTER(C.c_int)
    lib.fwi_init.argtypes = [I]
    lib.fwi_last_error.restype = C.c_char_p
    lib.fwi_set_stream.argtypes = [P]
    lib.fwi_set_solver_options.argtypes = [I, I]
    lib.fwi_kernel_launch_count.restype = C.c_int64
    lib.fwi_batch_plans.restype = C.c_int64
    lib.fwi_solver_acoustic_ss.argtypes = [P] * 21
    lib.fwi_misfit_function.argtypes = [P] * 10
    lib.fwi_beta_calculous.argtypes = [P] * 7
    lib.fwi_first_step.argtypes = [P] * 5
    lib.fwi_model_update.argtypes = [P] * 6
    lib.fwi_mcs_geometry.argtypes = [F, F, F, F, F, F, I, P, P, P, P]
    lib.fwi_ricker.argtypes = [F, F, I, P]
    lib.fwi_was_geometry.argtypes = [I, P, P, I, P, P, F, F, I, I, P, P, P, P, P, P]
    lib.fwi_time_rules.argtypes = [P, I, I, F, F, I, P, P, P]
    lib.fwi_survey_create.argtypes = [C.POINTER(FwiSurveyDesc), C.POINTER(C.c_void_p)]
    lib.fwi_survey_destroy.argtypes = [P]
    lib.fwi_survey_set_lambda.argtypes = [P, P]
    lib.fwi_survey_set_observed.argtypes = [P, P]
    lib.fwi_survey_set_sources.argtypes = [P, P]
    lib.fwi_survey_set_time.argtypes = [P, F, I, P, P]
    lib.fwi_time_filter.argtypes = [P] * 7
    lib.fwi_set_filter_order.argtypes = [I]
    lib.fwi_interpolation_akima.argtypes = [P] * 7
    lib.fwi_su_info.argtypes = [C.c_char_p, I, P, P, P]
    lib.fwi_su_read.argtypes = [C.c_char_p, I, I, I, P]
    lib.fwi_su_write.argtypes = [C.c_char_p, P, I, I, F, I]
    lib.fwi_read_nav.argtypes = [C.c_char_p, I, P, P, P, P]
    lib.fwi_su_supershot.argtypes = [C.POINTER(C.c_char_p), I, P, I, I, I, P]
    lib.fwi_survey_run.argtypes = [P, I, P, P]
    lib.fwi_survey_grad_device.argtypes = [P, C.POINTER(C.c_void_p)]
    lib.fwi_survey_get_stack.argtypes = [P, C.c_void_p]
    lib.fwi_survey_get_synthetic.argtypes = [P, I, P]
    lib.fwi_survey_step_bytes.argtypes = [P, C.POINTER(C.c_double)]
    lib.fwi_survey_two_step_bytes.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.fwi_survey_tuning.argtypes = [P, IP, IP]
    lib.fwi_survey_recompute.argtypes = [P, IP, IP]
    lib.fwi_survey_tiles.argtypes = [P, IP, IP, P, P, IP]
    lib.fwi_survey_edge_tiles.argtypes = [P, IP, P, P, IP]
    lib.fwi_survey_launch_form.argtypes = [P, I, IP, C.POINTER(F), C.POINTER(F)]
    lib.fwi_survey_stepping.argtypes = [P, IP, C.POINTER(F), C.POINTER(F), C.POINTER(F)]
    lib.fwi_batch_survey.argtypes = [C.POINTER(C.c_void_p)]
    lib.fwi_survey_time_steps.argtypes = [P, I]
    lib.fwi_misfit_gradient_batch.argtypes = [C.POINTER(FwiSurveyDesc), P, I, P, P]
    lib.fwi_solver_forward_noalloc.argtypes = [I, I, P, P, P, P, P, F, F, I, I, P, I, P]
    for name in EXPORTS:
        fn = getattr(lib, name)
        if fn.restype is None and name not in ("fwi_last_error", "fwi_kernel_launch_count", "fwi_batch_plans"):
            fn.restype = C.c_int
    _lib = lib
    return lib


def check(rc):
    if rc != FWI_OK:
        msg = load().fwi_last_error()
        raise FwiError(rc, msg.decode() if msg else "")
    return rc
