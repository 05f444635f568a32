"""ctypes binding of libhyk.so (the C ABI declared in include/hyk.h).

The library is built in-tree by ``hyk._build.build()``.  There is no CPU
fallback: if the library is missing or cannot be loaded every GPU entry point
raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

from .decompose import hyk_decomp_t

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libhyk.so")
_lock = threading.Lock()
_lib = None

P = ctypes.POINTER
c_u32, c_u64, c_i64, c_int, c_d, c_vp = (
    ctypes.c_uint32,
    ctypes.c_uint64,
    ctypes.c_int64,
    ctypes.c_int,
    ctypes.c_double,
    ctypes.c_void_p,
)

HYK_MODE_PLAIN = 0
HYK_MODE_PERSISTENT = 1
HYK_ERR_INVALID = -1
HYK_ERR_CUDA = -2
HYK_ERR_NVRTC = -3
HYK_ERR_UNSUPPORTED = -4
HYK_ERR_TIMEOUT = -5

HYK_CFG_PIN_ARITH = 1
HYK_CFG_ADJOINT = 2
HYK_CFG_HIGH_ACCURACY = 4
HYK_CFG_GLOBAL_JETS = 8
HYK_CFG_FLOAT32 = 16
HYK_CFG_NO_COLD_ROWS = 32
HYK_CFG_DEBUG = 64
HYK_DBG_LANE_RANGE = 1
HYK_DBG_NONFINITE_JET = 2
HYK_DBG_CAPACITY = 4

LANE_DONE, LANE_STOPPED, LANE_CAPACITY, LANE_EVENT = 1, 2, 4, 8
OC_EV_OVERFLOW = -4294967310


class hyk_config_t(ctypes.Structure):
    _fields_ = [
        ("block_lanes", c_u32),
        ("persist_ctas", c_u32),
        ("flags", c_u32),
        ("team_size", c_u32),
    ]


class hyk_module_info_t(ctypes.Structure):
    _fields_ = [
        ("n_eq", c_u32),
        ("n_pars", c_u32),
        ("order", c_u32),
        ("n_u", c_u32),
        ("block_lanes", c_u32),
        ("smem_per_lane", c_u32),
        ("regs_per_thread", c_u32),
        ("ctas_per_sm", c_u32),
        ("n_sm", c_u32),
        ("reserved", c_u32),
        ("flops_per_step", c_d),
        ("compile_seconds", c_d),
        ("team_size", c_u32),
        ("reserved2", c_u32),
    ]


class hyk_lanes_t(ctypes.Structure):
    _fields_ = [
        ("n_lanes", c_u64),
        ("ld", c_u64),
        ("state", c_vp),
        ("pars", c_vp),
        ("time_hi", c_vp),
        ("time_lo", c_vp),
    ]


class hyk_prop_t(ctypes.Structure):
    _fields_ = [
        ("tf_hi", c_vp),
        ("tf_lo", c_vp),
        ("max_delta_t", c_vp),
        ("max_steps", c_u64),
        ("grid", c_vp),
        ("n_grid", c_u64),
        ("grid_out", c_vp),
        ("tc_out", c_vp),
        ("tc_t_hi", c_vp),
        ("tc_t_lo", c_vp),
        ("tc_capacity", c_u64),
        ("rem_hi", c_vp),
        ("rem_lo", c_vp),
        ("outcome", c_vp),
        ("min_h", c_vp),
        ("max_h", c_vp),
        ("n_steps", c_vp),
        ("n_iter", c_vp),
        ("grid_idx", c_vp),
        ("last_h", c_vp),
        ("last_tc", c_vp),
        ("status", c_vp),
        ("lane_order", c_vp),
        ("n_order", c_u64),
        ("ck_x", c_vp),
        ("ck_t", c_vp),
        ("ck_h", c_vp),
        ("ck_capacity", c_u64),
        ("slice_iters", c_u64),
        ("ev_t_hi", c_vp),
        ("ev_t_lo", c_vp),
        ("ev_info", c_vp),
        ("ev_count", c_vp),
        ("ev_capacity", c_u64),
        ("ev_last", c_vp),
        ("ev_sign", c_vp),
        ("stop_iter", c_vp),
        ("stop_group", c_u64),
    ]


class hyk_serve_t(ctypes.Structure):
    _fields_ = [
        ("ring", c_vp),
        ("ring_capacity", c_u64),
        ("head", c_vp),
        ("tail", c_vp),
        ("stop", c_vp),
        ("owner", c_vp),
        ("done_count", c_vp),
        ("inflight", c_vp),
        ("status", c_vp),
        ("idle_ns", c_u64),
        ("max_wait_ns", c_u64),
        ("grid_ctas", c_u32),
    ]


HYK_SERVE_IDLE, HYK_SERVE_STOP, HYK_SERVE_TIMEOUT = 1, 2, 4


# Every function the header declares, with its ctypes signature.
SIGNATURES = {
    "hyk_module_create": (c_int, [P(hyk_decomp_t), c_u32, P(hyk_config_t), c_int, P(c_vp)]),
    "hyk_module_destroy": (c_int, [c_vp]),
    "hyk_module_get_info": (c_int, [c_vp, P(hyk_module_info_t)]),
    "hyk_module_source": (ctypes.c_char_p, [c_vp]),
    "hyk_module_debug": (c_int, [c_vp, c_vp, c_int]),
    "hyk_step": (c_int, [c_vp, P(hyk_lanes_t), c_vp, c_int, c_vp, c_vp, c_vp, P(hyk_prop_t), c_vp]),
    "hyk_prop_init": (c_int, [c_vp, P(hyk_lanes_t), P(hyk_prop_t), c_vp]),
    "hyk_propagate_workspace_size": (ctypes.c_size_t, [c_vp, c_u64, c_int]),
    "hyk_propagate": (
        c_int,
        [c_vp, P(hyk_lanes_t), P(hyk_prop_t), c_int, c_vp, ctypes.c_size_t, c_u32, P(c_u64), c_vp],
    ),
    "hyk_propagate_noalloc": (c_int, [c_vp, P(hyk_lanes_t), P(hyk_prop_t), c_int, c_u32, P(c_u64), c_vp]),
    "hyk_adjoint": (c_int, [c_vp, P(hyk_lanes_t), c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_size_t, c_vp]),
    "hyk_dense_eval": (c_int, [c_vp, c_u32, c_u32, c_u64, c_u64, c_vp, c_vp, c_vp]),
    "hyk_dense_eval_f32": (c_int, [c_vp, c_u32, c_u32, c_u64, c_u64, c_vp, c_vp, c_vp]),
    "hyk_fp64_peak": (c_int, [c_int, c_d, P(c_d)]),
    "hyk_fp32_peak": (c_int, [c_int, c_d, P(c_d)]),
    "hyk_dmath_eval": (c_int, [c_int, c_vp, c_vp, c_vp, c_u64, c_vp]),
    "hyk_serve": (c_int, [c_vp, P(hyk_lanes_t), P(hyk_prop_t), P(hyk_serve_t), c_vp]),
    "hyk_memcpy2d": (c_int, [c_vp, ctypes.c_size_t, c_vp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, c_vp]),
    "hyk_codegen_check": (
        c_int,
        [P(hyk_decomp_t), c_u32, P(hyk_config_t), c_int, ctypes.c_char_p, ctypes.c_size_t, P(c_u32), P(c_d)],
    ),
    "hyk_last_error": (ctypes.c_char_p, []),
    "hyk_version": (ctypes.c_char_p, []),
}


class HykError(RuntimeError):
    pass


def lib_path() -> str:
    return _LIB_PATH


def load():
    """Load libhyk.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                raise HykError(
                    "libhyk.so is not built ({}); run hyk._build.build() or "
                    "__graft_entry__.build() first".format(_LIB_PATH)
                )
            L = ctypes.CDLL(_LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = load().hyk_last_error().decode(errors="replace")
        raise HykError("{}{}".format(what + ": " if what else "", msg))
