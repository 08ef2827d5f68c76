"""GB300-native FWI hot path: per-shot forward/adjoint acoustic propagation,
L2 misfit and adjoint source, imaging condition and gradient stack, as
hand-written sm_103a kernels behind the C ABI of include/fwi_gb300.h.

Every entry point loads fwi_gb300/_lib/libfwi_gb300.so and raises if it is
missing (build it with ``python -m fwi_gb300.build``): there is no CPU
fallback.
"""
from ._native import (  # noqa: F401
    GRAD_F32,
    GRAD_F64,
    SNAP_BF16,
    SNAP_F16,
    SNAP_F32,
    SURVEY_NO_GRAPH,
    SURVEY_RECOMPUTE,
    SURVEY_SINGLE_STEP,
    SURVEY_FUSED_STEP,
    SURVEY_GRAPH,
    FwiError,
    load,
)
from .survey import ShotSpec, SurveySpec  # noqa: F401

from .api import (  # noqa: E402,F401
    Beta_calculous,
    Misfit_function,
    Ricker_mcs,
    Survey,
    batch_release,
    batch_survey,
    calculate_misfit_gradient,
    first_step,
    init,
    interpolation_akima,
    kernel_launch_count,
    mcs_geometry,
    model_update,
    read_nav,
    set_filter_order,
    set_solver_options,
    set_stream,
    solver_acoustic_SS,
    su_info,
    su_read,
    su_supershot,
    su_write,
    time_filter,
    time_rules,
    was_geometry,
)
