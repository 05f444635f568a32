"""GPU module cache and thin wrappers over the C ABI (device pointers in, status out)."""

from __future__ import annotations

import ctypes
import threading

import torch

from . import _lib
from .decompose import Decomposition

_cache_lock = threading.Lock()
_modules: dict = {}


class Module:
    """A compiled (decomposition, order, config) on one device; shared by integrators."""

    def __init__(self, dec: Decomposition, order: int, device: int, block_lanes: int = 0, pin_arith: bool = False,
                 team_size: int = 0, persist_ctas: int = 0, high_accuracy: bool = False, global_jets: bool = False,
                 float32: bool = False, cold_rows: bool = True, debug: bool = False):
        L = _lib.load()
        self.dec, self.order, self.device = dec, int(order), int(device)
        self._cdec, self._keep = dec.as_c()
        flags = (_lib.HYK_CFG_PIN_ARITH if pin_arith else 0) | (_lib.HYK_CFG_HIGH_ACCURACY if high_accuracy else 0)
        flags |= _lib.HYK_CFG_GLOBAL_JETS if global_jets else 0
        flags |= _lib.HYK_CFG_FLOAT32 if float32 else 0
        flags |= 0 if cold_rows else _lib.HYK_CFG_NO_COLD_ROWS
        flags |= _lib.HYK_CFG_DEBUG if debug else 0
        self.debug = bool(debug)
        self.float32 = bool(float32)
        cfg = _lib.hyk_config_t(int(block_lanes), int(persist_ctas), flags, int(team_size))
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.current_stream().synchronize()
            _lib.check(
                L.hyk_module_create(ctypes.byref(self._cdec), self.order, ctypes.byref(cfg), self.device, ctypes.byref(h)),
                "hyk_module_create",
            )
        self.handle = h
        info = _lib.hyk_module_info_t()
        _lib.check(L.hyk_module_get_info(h, ctypes.byref(info)))
        self.info = info
        self.ws = torch.zeros(64, dtype=torch.int32, device=torch.device("cuda", self.device))
        self.ws_bytes = int(L.hyk_propagate_workspace_size(h, 0, 1))
        if self.ws.data_ptr() % 256 != 0:  # pragma: no cover - torch allocations are 512-byte aligned
            raise _lib.HykError("workspace misaligned")

    def close(self):
        """Unload the module and free its device buffers (after its last use)."""
        h, self.handle = getattr(self, "handle", None), None
        if h is not None and h.value:
            torch.cuda.synchronize(self.device)  # no launch of the module may still be running
            _lib.load().hyk_module_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown: nothing left to free
            pass

    def debug_record(self, clear: bool = False):
        """The debug record of a module built with ``debug=True`` (the
        device synchronised first): the codes seen, the number of findings
        and the first one."""
        import numpy as np

        torch.cuda.synchronize(self.device)
        out = np.zeros(8, dtype=np.uint64)
        _lib.check(_lib.load().hyk_module_debug(self.handle, out.ctypes.data, int(bool(clear))), "hyk_module_debug")
        names = {_lib.HYK_DBG_LANE_RANGE: "lane_range", _lib.HYK_DBG_NONFINITE_JET: "nonfinite_jet",
                 _lib.HYK_DBG_CAPACITY: "capacity"}
        codes = int(out[0])
        rec = {"codes": [n for c, n in names.items() if codes & c], "count": int(out[1]), "first": None}
        if out[1]:
            c = int(out[2])
            d = [int(x) for x in out[3:7]]
            keys = {_lib.HYK_DBG_LANE_RANGE: ("index", "n_lanes", "position", None),
                    _lib.HYK_DBG_NONFINITE_JET: ("lane", "variable", "order", "iteration"),
                    _lib.HYK_DBG_CAPACITY: ("lane", "iteration", None, None)}.get(c, ("a", "b", "c", "d"))
            rec["first"] = dict({"code": names.get(c, str(c))}, **{k: v for k, v in zip(keys, d) if k})
        return rec

    @property
    def source(self) -> str:
        return _lib.load().hyk_module_source(self.handle).decode()

    def info_dict(self):
        i = self.info
        return {
            "n_eq": i.n_eq,
            "n_pars": i.n_pars,
            "order": i.order,
            "n_u": i.n_u,
            "block_lanes": i.block_lanes,
            "smem_per_lane": i.smem_per_lane,
            "regs_per_thread": i.regs_per_thread,
            "ctas_per_sm": i.ctas_per_sm,
            "n_sm": i.n_sm,
            "local_bytes": i.reserved,
            "flops_per_step": i.flops_per_step,
            "compile_seconds": i.compile_seconds,
            "team_size": i.team_size,
        }


def get_module(dec: Decomposition, order: int, device: int, block_lanes: int = 0, pin_arith: bool = False,
               team_size: int = 0, persist_ctas: int = 0, high_accuracy: bool = False,
               global_jets: bool = False, float32: bool = False, cold_rows: bool = True, debug: bool = False) -> Module:
    key = (dec.digest(), int(order), int(device), int(block_lanes), bool(pin_arith), int(team_size), int(persist_ctas),
           bool(high_accuracy), bool(global_jets), bool(float32), bool(cold_rows), bool(debug))
    with _cache_lock:
        m = _modules.get(key)
        if m is None:
            m = Module(dec, order, device, block_lanes, pin_arith, team_size, persist_ctas, high_accuracy, global_jets,
                       float32, cold_rows, debug)
            _modules[key] = m
        return m


def drop_modules(keep=()):
    """Forget the cached modules except those in ``keep``: each is unloaded
    (and its device buffers freed) when no integrator uses it any more."""
    keep_ids = {id(m) for m in keep}
    with _cache_lock:
        for k in [k for k, m in _modules.items() if id(m) not in keep_ids]:
            del _modules[k]


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def lanes_struct(state, pars, t_hi, t_lo):
    B = state.shape[1]
    return _lib.hyk_lanes_t(
        B,
        state.stride(0) if state.dim() == 2 else B,
        state.data_ptr(),
        pars.data_ptr() if pars is not None and pars.numel() > 0 else None,
        t_hi.data_ptr(),
        t_lo.data_ptr(),
    )


def stream_handle(device: int):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
