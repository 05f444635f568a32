"""Differentiable propagation: the discrete adjoint of the Taylor integrator.

``taylor_flow(sys, x0, t_final, pars=None, tol=0.0)`` propagates every lane
from its initial state to ``t_final`` with the persistent kernel and returns
the final state as a torch tensor that is differentiable with respect to
``x0`` and ``pars`` (``torch.autograd``).

Forward: the usual propagation, plus a per-step tape of the state, time and
step size at the start of every step (grown and resumed when a lane fills
it).  Backward: libhyk's adjoint kernel walks each lane's tape backwards,
recomputes the step's Taylor coefficients from the taped state and applies
the transpose of the step's Jacobian — the reverse sweep through the Horner
update and every Taylor recurrence — with the taped step sizes held fixed.
The result is the exact gradient of the discrete map the forward pass
applied (a step-size change moves the solution only at the tolerance level),
checked against central finite differences and against first-order
variational equations (``var_ode_sys``) in the tests.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .core import get_module, lanes_struct, stream_handle
from .decompose import order_from_tol, taylor_decompose

EPS = 2.220446049250313e-16
# The reverse sweep takes its lanes longest tape first (the order changes the
# schedule only, never a lane's arithmetic).
LONGEST_FIRST = True


def _propagate_taped(mod, x, pars, t0, tf, cap=64):
    """Propagate lanes (x: (n_eq, B)) from t0 to tf (B,), taping every step."""
    L = _lib.load()
    dev = x.device
    ne, B = x.shape
    f64 = dict(dtype=torch.float64, device=dev)
    th = t0.clone().contiguous()
    tl = torch.zeros(B, **f64)
    a = {
        "rem_hi": torch.empty(B, **f64), "rem_lo": torch.empty(B, **f64),
        "outcome": torch.empty(B, dtype=torch.int64, device=dev), "min_h": torch.empty(B, **f64),
        "max_h": torch.empty(B, **f64), "n_steps": torch.empty(B, dtype=torch.int64, device=dev),
        "n_iter": torch.empty(B, dtype=torch.int64, device=dev), "last_h": torch.empty(B, **f64),
        "status": torch.empty(B, dtype=torch.int32, device=dev),
    }
    ck_x = torch.empty((cap, ne, B), **f64)
    ck_t = torch.empty((cap, B), **f64)
    ck_h = torch.empty((cap, B), **f64)

    def desc():
        return _lib.hyk_prop_t(
            tf.data_ptr(), None, None, 0, None, 0, None, None, None, None, 0,
            a["rem_hi"].data_ptr(), a["rem_lo"].data_ptr(), a["outcome"].data_ptr(), a["min_h"].data_ptr(),
            a["max_h"].data_ptr(), a["n_steps"].data_ptr(), a["n_iter"].data_ptr(), None, a["last_h"].data_ptr(),
            None, a["status"].data_ptr(), None, 0, ck_x.data_ptr(), ck_t.data_ptr(), ck_h.data_ptr(), cap, 0,
        )

    lanes = lanes_struct(x, pars, th, tl)
    with torch.cuda.device(dev):
        s = stream_handle(dev.index)
        _lib.check(L.hyk_prop_init(mod.handle, lanes, desc(), s), "hyk_prop_init")
        while True:
            _lib.check(
                L.hyk_propagate(mod.handle, lanes, desc(), _lib.HYK_MODE_PERSISTENT, mod.ws.data_ptr(), mod.ws_bytes,
                                0, None, s),
                "hyk_propagate",
            )
            full = (a["status"] & _lib.LANE_CAPACITY) != 0
            if not bool(full.any()):
                break
            ncap = 2 * cap
            nx, nt, nh = torch.empty((ncap, ne, B), **f64), torch.empty((ncap, B), **f64), torch.empty((ncap, B), **f64)
            nx[:cap], nt[:cap], nh[:cap] = ck_x, ck_t, ck_h
            ck_x, ck_t, ck_h, cap = nx, nt, nh, ncap
            a["status"] &= ~(_lib.LANE_CAPACITY | _lib.LANE_STOPPED)
    return x, th, a, ck_x, ck_t, ck_h


class _TaylorFlow(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, pars, fwd_mod, adj_mod, t0, tf):
        x = x0.detach().clone().contiguous()
        p = pars.detach().contiguous() if pars is not None else None
        x, th, a, ck_x, ck_t, ck_h = _propagate_taped(fwd_mod, x, p, t0, tf)
        ctx.adj_mod = adj_mod
        ctx.has_pars = pars is not None
        ctx.save_for_backward(ck_x, ck_t, ck_h, a["n_iter"], p if p is not None else torch.empty(0))
        ctx.mark_non_differentiable(th)
        ctx.res = {k: v for k, v in a.items()}
        return x, th

    @staticmethod
    def backward(ctx, gx, gt):
        ck_x, ck_t, ck_h, n_iter, p = ctx.saved_tensors
        mod = ctx.adj_mod
        L = _lib.load()
        lam = gx.detach().to(torch.float64).contiguous().clone()
        B = lam.shape[1]
        npar = mod.dec.n_pars
        pbar = torch.zeros((max(npar, 1), B), dtype=torch.float64, device=lam.device)
        dummy_t = torch.zeros(B, dtype=torch.float64, device=lam.device)
        lanes = lanes_struct(lam, p if ctx.has_pars else None, dummy_t, dummy_t)
        with torch.cuda.device(lam.device):
            # longest tape first: the last lanes taken are the short ones
            order = torch.argsort(n_iter, descending=True) if LONGEST_FIRST else None
            _lib.check(
                L.hyk_adjoint(mod.handle, lanes, ck_x.data_ptr(), ck_t.data_ptr(), ck_h.data_ptr(), n_iter.data_ptr(),
                              order.data_ptr() if order is not None else None, lam.data_ptr(),
                              pbar.data_ptr() if npar else None, mod.ws.data_ptr(), mod.ws_bytes,
                              stream_handle(lam.device.index)),
                "hyk_adjoint",
            )
            del order
        return lam, (pbar[:npar] if ctx.has_pars else None), None, None, None, None


def taylor_flow(sys, x0, t_final, pars=None, tol=0.0, t0=0.0):
    """Differentiable propagation of every lane of ``x0`` (torch, (n_eq, B),
    float64, CUDA) to ``t_final`` (scalar or (B,)); returns
    ``(state, time)`` with ``state`` differentiable with respect to ``x0``
    and ``pars`` ((n_pars, B))."""
    dec = taylor_decompose(sys)
    order = order_from_tol(tol if tol else EPS)
    dev = x0.device
    if dev.type != "cuda":
        raise ValueError("taylor_flow needs CUDA tensors")
    fwd = get_module(dec, order, dev.index)
    adj = _adjoint_module(dec, order, dev.index)
    B = x0.shape[1]
    f64 = dict(dtype=torch.float64, device=dev)
    tf = torch.as_tensor(t_final, **f64).expand(B).contiguous()
    tt0 = torch.as_tensor(t0, **f64).expand(B).contiguous()
    if pars is None and dec.n_pars:
        raise ValueError("the system has parameters: pass pars of shape (n_pars, batch)")
    return _TaylorFlow.apply(x0, pars, fwd, adj, tt0, tf)


_adj_cache = {}


def _adjoint_module(dec, order, device):
    from .core import Module

    key = (dec.digest(), order, device)
    m = _adj_cache.get(key)
    if m is None:
        m = _AdjModule(dec, order, device)
        _adj_cache[key] = m
    return m


class _AdjModule:
    def __init__(self, dec, order, device):
        L = _lib.load()
        self.dec, self.order, self.device = dec, order, device
        self._cdec, self._keep = dec.as_c()
        cfg = _lib.hyk_config_t(0, 0, _lib.HYK_CFG_ADJOINT, 0)
        h = ctypes.c_void_p()
        with torch.cuda.device(device):
            torch.cuda.current_stream().synchronize()
            _lib.check(L.hyk_module_create(ctypes.byref(self._cdec), order, ctypes.byref(cfg), device, ctypes.byref(h)),
                       "hyk_module_create (adjoint)")
        self.handle = h
        self.ws = torch.zeros(64, dtype=torch.int32, device=torch.device("cuda", device))
        self.ws_bytes = 256
