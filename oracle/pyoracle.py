"""ctypes front-end of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product path (the ``hyk`` package and libhyk.so) never does.
See hyk_oracle.cpp for the restated algorithm and its reference citations.

All arrays are float64 NumPy arrays in the reference's [var][lane] layout.
``prec``: 0 = double, 1 = binary128, 2 = float (gpu arithmetic).  ``mode``: 0 = "pin" arithmetic (the
arithmetic pinned to the reference's notebook outputs), 1 = "gpu" arithmetic
(fused multiply-adds and reciprocal multiplications, operation for operation
what the CUDA kernels do).
"""

from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if os.path.join(ROOT, "heyoka.py_gb300") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "heyoka.py_gb300"))

from hyk.decompose import hyk_decomp_t, taylor_decompose  # noqa: E402

_lib = None

P = ctypes.POINTER
c_d = ctypes.c_double
pd = P(c_d)
pi64 = P(ctypes.c_int64)
pu64 = P(ctypes.c_uint64)


def lib():
    global _lib
    if _lib is None:
        sys.path.insert(0, HERE)
        import build as _b  # oracle/build.py

        path = _b.build()
        L = ctypes.CDLL(path)
        L.hyko_last_error.restype = ctypes.c_char_p
        L.hyko_step.argtypes = [
            P(hyk_decomp_t), ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
            pd, pd, pd, pd, pd, ctypes.c_int, pi64, pd, pd,
        ]
        L.hyko_propagate.argtypes = [
            P(hyk_decomp_t), ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
            pd, pd, pd, pd, pd, pd, ctypes.c_uint64, pd, pd, ctypes.c_uint64, pd,
            ctypes.c_int, P(pd), P(pd), P(pd), pu64, pi64, pd, pd, pu64, pd, pd, pu64,
        ]
        L.hyko_ensemble_until.argtypes = [
            P(hyk_decomp_t), ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64,
            pd, pd, pd, pd, pd, ctypes.c_int, pi64, pd, pd, pu64, ctypes.c_int,
        ]
        L.hyko_propagate_ev.argtypes = [
            P(hyk_decomp_t), ctypes.c_uint32, ctypes.c_uint32, pd, pd, pd, pd, pd, ctypes.c_uint64, pi64, pu64,
            P(ctypes.c_uint32), pd, P(ctypes.c_int32), pu64, P(pd), P(pd), P(P(ctypes.c_int32)),
            P(P(ctypes.c_uint32)), ctypes.c_int,
        ]
        L.hyko_ev_find.argtypes = [pd, ctypes.c_uint32, c_d, c_d, c_d, ctypes.c_int, ctypes.c_int, pd,
                                   P(ctypes.c_int32), ctypes.c_int]
        L.hyko_free.argtypes = [ctypes.c_void_p]
        L.hyko_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, t=pd):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Oracle:
    """A batch of B lanes of one ODE system, integrated on the CPU."""

    def __init__(self, sys_or_dec, state, pars=None, time=None, order=20, prec=0, mode=0):
        self.dec = sys_or_dec if hasattr(sys_or_dec, "ops") else taylor_decompose(sys_or_dec)
        self.cdec, self._keep = self.dec.as_c()
        self.state = _f64(state).copy()
        if self.state.ndim != 2 or self.state.shape[0] != self.dec.n_eq:
            raise ValueError("state must have shape (n_eq, B)")
        self.B = self.state.shape[1]
        npar = max(self.dec.n_pars, 0)
        self.pars = (
            np.zeros((npar, self.B)) if pars is None else _f64(pars).reshape(npar, self.B).copy()
        )
        self.t_hi = np.zeros(self.B) if time is None else _f64(np.broadcast_to(time, (self.B,))).copy()
        self.t_lo = np.zeros(self.B)
        self.order, self.prec, self.mode = int(order), int(prec), int(mode)
        self.last_h = np.zeros(self.B)
        self.tc = np.zeros((self.dec.n_eq, self.order + 1, self.B))

    def _err(self, rc):
        if rc != 0:
            raise RuntimeError(lib().hyko_last_error().decode())

    def step(self, max_delta_t=None, backward=False, write_tc=True):
        B = self.B
        oc = np.zeros(B, dtype=np.int64)
        h = np.zeros(B)
        md = None if max_delta_t is None else _f64(np.broadcast_to(max_delta_t, (B,))).copy()
        rc = lib().hyko_step(
            ctypes.byref(self.cdec), self.order, self.prec, self.mode, B,
            _p(self.state), _p(self.pars) if self.pars.size else None, _p(self.t_hi), _p(self.t_lo),
            _p(md), int(bool(backward)), _p(oc, pi64), _p(h), _p(self.tc),
        )
        self._err(rc)
        self.last_h = h.copy()
        return oc, h

    def propagate_until(self, t, max_steps=0, max_delta_t=None, c_output=False, t_lo=None):
        B = self.B
        tf = _f64(np.broadcast_to(t, (B,))).copy()
        tfl = None if t_lo is None else _f64(np.broadcast_to(t_lo, (B,))).copy()
        return self._prop(tf, tfl, max_steps, max_delta_t, None, c_output)

    def propagate_for(self, delta_t, max_steps=0, max_delta_t=None, c_output=False):
        # target = time + delta_t in double-length arithmetic
        dt = _f64(np.broadcast_to(delta_t, (self.B,)))
        hi, lo = _dadd(self.t_hi, self.t_lo, dt, np.zeros_like(dt))
        return self._prop(hi, lo, max_steps, max_delta_t, None, c_output)

    def propagate_grid(self, grid, max_steps=0, max_delta_t=None):
        grid = _f64(grid)
        if grid.ndim != 2 or grid.shape[1] != self.B:
            raise ValueError("grid must have shape (n, B)")
        tf = grid[-1].copy()
        return self._prop(tf, None, max_steps, max_delta_t, grid, False)

    def _prop(self, tf, tfl, max_steps, max_delta_t, grid, c_output):
        B, ne, p = self.B, self.dec.n_eq, self.order
        oc = np.zeros(B, dtype=np.int64)
        mn, mx, lh = np.zeros(B), np.zeros(B), np.zeros(B)
        ns = np.zeros(B, dtype=np.uint64)
        nit = ctypes.c_uint64(0)
        cn = ctypes.c_uint64(0)
        md = None if max_delta_t is None else _f64(np.broadcast_to(max_delta_t, (B,))).copy()
        gout = None
        if grid is not None:
            gout = np.zeros((grid.shape[0], ne, B))
        c_t, c_h, c_l = pd(), pd(), pd()
        ltc = np.zeros((ne, p + 1, B))
        rc = lib().hyko_propagate(
            ctypes.byref(self.cdec), p, self.prec, self.mode, B,
            _p(self.state), _p(self.pars) if self.pars.size else None, _p(self.t_hi), _p(self.t_lo),
            _p(tf), _p(tfl), int(max_steps), _p(md),
            _p(grid), 0 if grid is None else grid.shape[0], _p(gout),
            int(bool(c_output)), ctypes.byref(c_t), ctypes.byref(c_h), ctypes.byref(c_l),
            ctypes.byref(nit), _p(oc, pi64), _p(mn), _p(mx), _p(ns, pu64), _p(lh), _p(ltc), ctypes.byref(cn),
        )
        self._err(rc)
        self.last_h = lh
        if nit.value > 0:
            self.tc = ltc
        res = {"outcome": oc, "min_h": mn, "max_h": mx, "n_steps": ns, "n_iter": nit.value, "grid": gout}
        if c_output:
            n = cn.value
            res["c_tcs"] = np.ctypeslib.as_array(c_t, shape=(max(n, 1) * ne * (p + 1) * B,))[
                : n * ne * (p + 1) * B
            ].reshape(n, ne, p + 1, B).copy()
            res["c_thi"] = np.ctypeslib.as_array(c_h, shape=((n + 1) * B,)).reshape(n + 1, B).copy()
            res["c_tlo"] = np.ctypeslib.as_array(c_l, shape=((n + 1) * B,)).reshape(n + 1, B).copy()
            for q in (c_t, c_h, c_l):
                lib().hyko_free(q)
        return res


def _two_sum(a, b):
    s = a + b
    bb = s - a
    e = (a - (s - bb)) + (b - bb)
    return s, e


def _dadd(xh, xl, yh, yl):
    s, e = _two_sum(xh, yh)
    e = e + (xl + yl)
    hi = s + e
    lo = e - (hi - s)
    return hi, lo


def ensemble_until(sys_or_dec, state, pars, t0, tf, order, batch=8, n_threads=0, mode=1, prec=0):
    """Ensemble of batch integrators of `batch` lanes each (OpenMP over
    batches); prec 0 double, 2 float."""
    dec = sys_or_dec if hasattr(sys_or_dec, "ops") else taylor_decompose(sys_or_dec)
    cdec, keep = dec.as_c()
    state = _f64(state).copy()
    n = state.shape[1]
    pars = np.zeros((dec.n_pars, n)) if pars is None else _f64(pars).reshape(dec.n_pars, n).copy()
    t_hi = _f64(np.broadcast_to(t0, (n,))).copy()
    t_lo = np.zeros(n)
    tfa = _f64(np.broadcast_to(tf, (n,))).copy()
    oc = np.zeros(n, dtype=np.int64)
    mn, mx = np.zeros(n), np.zeros(n)
    ns = np.zeros(n, dtype=np.uint64)
    rc = lib().hyko_ensemble_until(
        ctypes.byref(cdec), order, mode, batch, n, _p(state), _p(pars) if pars.size else None,
        _p(t_hi), _p(t_lo), _p(tfa), int(n_threads), _p(oc, pi64), _p(mn), _p(mx), _p(ns, pu64), int(prec),
    )
    if rc != 0:
        raise RuntimeError(lib().hyko_last_error().decode())
    return {"state": state, "t_hi": t_hi, "t_lo": t_lo, "outcome": oc, "min_h": mn, "max_h": mx, "n_steps": ns}


def ev_find(g, h, s_lo=0.0, s_hi=1.0, direction=0, first_only=False, maxr=256):
    """The kernels' event root finder (hyk_events.h) on the host: roots s in
    (s_lo, s_hi] of sum g_n (h s)^n, with their directions."""
    g = _f64(g)
    rs = np.zeros(maxr)
    rsg = np.zeros(maxr, dtype=np.int32)
    n = lib().hyko_ev_find(_p(g), len(g) - 1, h, s_lo, s_hi, int(direction), int(first_only), _p(rs),
                           rsg.ctypes.data_as(P(ctypes.c_int32)), maxr)
    return rs[: min(n, maxr)], rsg[: min(n, maxr)], n


def propagate_ev(sys_, events, state, tf, pars=None, order=20, max_steps=0, time=None, ev_last=None, time_lo=None,
                 prec=0):
    """Per-lane propagation with events in gpu arithmetic, the kernels'
    semantics (prec 0 double, 2 float).  events: (expression, terminal,
    direction, cooldown) tuples in the integrator's order (terminal events first).  Returns a dict with
    state, t_hi, t_lo, outcome, n_steps, status, ev_last, ev_sign and the
    non-terminal records (rec_t_hi, rec_t_lo, rec_info, rec_lane)."""
    dec = taylor_decompose(sys_, events=events)
    cdec, keep = dec.as_c()
    st = _f64(state).copy()
    B = st.shape[1]
    pa = np.zeros((max(dec.n_pars, 1), B)) if pars is None else _f64(pars).reshape(-1, B).copy()
    th = np.zeros(B) if time is None else _f64(np.broadcast_to(time, (B,))).copy()
    tl = np.zeros(B) if time_lo is None else _f64(np.broadcast_to(time_lo, (B,))).copy()
    tfv = _f64(np.broadcast_to(tf, (B,))).copy()
    n_term = max(sum(1 for e in events if e[1]), 1)
    last = np.full((n_term, B), np.nan) if ev_last is None else _f64(ev_last).copy()
    sign = np.zeros(B, dtype=np.int32)
    oc = np.zeros(B, dtype=np.int64)
    ns = np.zeros(B, dtype=np.uint64)
    status = np.zeros(B, dtype=np.uint32)
    nrec = ctypes.c_uint64()
    rh, rl = pd(), pd()
    ri, rln = P(ctypes.c_int32)(), P(ctypes.c_uint32)()
    L = lib()
    rc = L.hyko_propagate_ev(ctypes.byref(cdec), order, B, _p(st), _p(pa), _p(th), _p(tl), _p(tfv), max_steps,
                             _p(oc, pi64), _p(ns, pu64), status.ctypes.data_as(P(ctypes.c_uint32)), _p(last),
                             sign.ctypes.data_as(P(ctypes.c_int32)), ctypes.byref(nrec), ctypes.byref(rh),
                             ctypes.byref(rl), ctypes.byref(ri), ctypes.byref(rln), int(prec))
    if rc != 0:
        raise RuntimeError(L.hyko_last_error().decode())
    n = nrec.value
    out = {
        "state": st, "t_hi": th, "t_lo": tl, "outcome": oc, "n_steps": ns, "status": status, "ev_last": last,
        "ev_sign": sign,
        "rec_t_hi": np.ctypeslib.as_array(rh, (max(n, 1),))[:n].copy(),
        "rec_t_lo": np.ctypeslib.as_array(rl, (max(n, 1),))[:n].copy(),
        "rec_info": np.ctypeslib.as_array(ri, (max(n, 1),))[:n].copy(),
        "rec_lane": np.ctypeslib.as_array(rln, (max(n, 1),))[:n].copy(),
    }
    for ptr in (rh, rl, ri, rln):
        L.hyko_free(ptr)
    return out
