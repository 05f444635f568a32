"""hyk - GB300-native batch Taylor integrator with heyoka.py's batch API.

The Python surface mirrors heyoka.py's (heyoka/__init__.py): expressions
(``make_vars``, ``par``, ``time``, elementary functions), the ``model``
factories, ``taylor_adaptive_batch``, ``taylor_outcome``,
``continuous_output_batch`` and the ``ensemble_propagate_*`` functions.  The
arithmetic runs in FP64 CUDA kernels generated per ODE system and compiled
with NVRTC for sm_103a (libhyk.so, C ABI in include/hyk.h).
"""
from .expr import expression, make_vars, par, time, sin, cos, exp, log, sqrt, square, sum, prod  # noqa: F401
from .decompose import taylor_decompose, order_from_tol  # noqa: F401
from .expr import diff  # noqa: F401
from .var import var_args, var_ode_sys  # noqa: F401
from . import callback, model, workloads  # noqa: F401
from .integrator import code_model, taylor_adaptive_batch, taylor_outcome  # noqa: F401
from .events import event_direction, nt_event, nt_event_batch, t_event, t_event_batch  # noqa: F401
from .c_output import continuous_output_batch, continuous_output_batch_dbl, continuous_output_batch_flt  # noqa: F401
from .s11n import get_serialization_backend, set_serialization_backend  # noqa: F401
from .scalar import continuous_output, continuous_output_dbl, continuous_output_flt, taylor_adaptive  # noqa: F401
from .ensemble import (  # noqa: F401
    ensemble_propagate_for,
    ensemble_propagate_for_batch,
    ensemble_propagate_grid,
    ensemble_propagate_grid_batch,
    ensemble_propagate_until,
    ensemble_propagate_until_batch,
)


def recommended_simd_size(fp_type=float):
    """Lanes per batch for good GPU occupancy (the reference returns the CPU SIMD width)."""
    return 32


def fp64_peak(device=0, millis=200.0):
    """Measured FP64 FMA throughput of the device in flop/s (2 flops per FMA)."""
    import ctypes

    from . import _lib

    v = ctypes.c_double()
    _lib.check(_lib.load().hyk_fp64_peak(int(device), float(millis), ctypes.byref(v)), "hyk_fp64_peak")
    return v.value


def fp32_peak(device=0, millis=200.0):
    """Measured FP32 FMA throughput of the device in flop/s (2 flops per FMA)."""
    import ctypes

    from . import _lib

    v = ctypes.c_double()
    _lib.check(_lib.load().hyk_fp32_peak(int(device), float(millis), ctypes.byref(v)), "hyk_fp32_peak")
    return v.value
