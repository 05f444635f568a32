"""``taylor_adaptive_batch``: the reference's batch integrator API on the GPU.

Mirrors the Python surface of heyoka.py's batch integrator
(heyoka/expose_batch_integrators.cpp:214-729, constructor at :91-212 and
:276-289, dispatch at heyoka/__init__.py:78-86): same constructor arguments,
methods, properties, return tuples and error messages.  Differences that
follow from living on a GPU:

* ``state`` and ``pars`` are writable **torch CUDA tensors** (shape
  ``(n, batch_size)``), not NumPy views; ``ta.state[:] = ...`` works as in the
  reference.  ``time``, ``dtime``, ``tc``, ``last_h``, ``d_output`` are
  read-only NumPy copies, as read-only as the reference's.
* ``batch_size`` is the number of GPU lanes: any size, not the SIMD width.
* ``fp_type`` is ``float`` (double precision) or ``numpy.float32`` (the
  reference's float batch integrator: float32 tensors, float kernels).  LLVM
  code-generation options are accepted and ignored.
* Step callbacks (``callback=``: one callable, an object with ``pre_hook``, or
  a list) run on the host after each batch step; the persistent kernel then
  advances every lane by one step per launch, so a propagation with a
  callback runs at one launch and one host round trip per step.  Events are
  detected on the device; with ``batch_semantics="reference"`` (the default)
  their callbacks run on the host after each batch step, as in the reference,
  and with ``"lane"`` when the propagation returns (``hyk/events.py``).
* ``propagate_*`` run every lane to its own final time in one persistent
  kernel launch (``prop_mode="persistent"``, the default), with one kernel
  launch per step over the lanes not yet finished (``prop_mode="plain"``), or
  with one launch per step over every lane (``prop_mode="plain_inplace"``:
  the reference's batch step called in a loop).  Per-lane results follow the
  reference's batch rules; the whole-batch rules that couple lanes are applied
  afterwards: a step limit reached by any lane gives ``step_limit`` to every
  lane, and lanes that finished before the batch's last iteration report
  ``last_h == 0`` and the Taylor coefficients of their final state (the zero
  steps the reference takes on them).  A state that becomes non-finite stops
  the whole batch at that iteration (``batch_semantics="reference"``) or only
  its own lane (``"lane"``).
"""

from __future__ import annotations

import copy as _copy
import enum
import math
import warnings

import numpy as np
import torch

from . import _lib
from .core import get_module, lanes_struct, stream_handle
from .decompose import order_from_tol, taylor_decompose

_PROP_MODES = ("persistent", "plain", "plain_inplace")

EPS = float(np.finfo(np.float64).eps)


def _fp_of(fp_type):
    """(NumPy dtype, torch dtype) of a supported floating-point type (the
    reference's dispatch: heyoka/__init__.py:55-86)."""
    if fp_type in (float, np.float64):
        return np.float64, torch.float64
    if fp_type is np.float32:
        return np.float32, torch.float32
    raise TypeError('The floating-point type "{}" is not recognized/supported'.format(fp_type))


class taylor_outcome(enum.IntEnum):
    """Outcome of a step or propagation (values of heyoka/core.cpp:324-329)."""

    success = -4294967297
    step_limit = -4294967298
    time_limit = -4294967299
    err_nf_state = -4294967300
    cb_stop = -4294967301

    @classmethod
    def _missing_(cls, value):
        # Terminal events: a step reports the event's index k >= 0, a
        # propagation stopped by it reports -k - 1.
        if isinstance(value, int) and value > cls.success:
            pseudo = int.__new__(cls, value)
            pseudo._name_ = "terminal_event_{}".format(value if value >= 0 else -value - 1)
            pseudo._value_ = value
            return cls._value2member_map_.setdefault(value, pseudo)
        return None


_LLVM_KWARGS = ("opt_level", "force_avx512", "slp_vectorize", "fast_math", "code_model", "parjit")


class code_model(enum.IntEnum):
    """LLVM code models, accepted for compatibility (heyoka/core.cpp code_model)."""

    tiny = 0
    small = 1
    kernel = 2
    medium = 3
    large = 4


class _LLVMStateInfo:
    """What ``llvm_state`` reports for a GPU integrator: the LLVM options it
    was constructed with (they do not affect the CUDA code), and the
    generated CUDA source in place of the IR."""

    def __init__(self, ta, opts):
        self._ta = ta
        self.__dict__.update(opts)

    def get_ir(self):
        return self._ta._mod.source

    def __repr__(self):
        return "GPU module (NVRTC, sm_103a); LLVM options: {}".format(
            {k: v for k, v in self.__dict__.items() if not k.startswith("_")})


def _to_fp_array(x, what, dt=np.float64):
    """x as a NumPy array of dtype dt: lossless conversions only for double,
    rounding to the nearest float for single precision."""
    a = np.asarray(x)
    if a.dtype != dt:
        a = a.astype(dt, casting="safe" if dt == np.float64 else "same_kind")
    return a


def _is_scalar(x):
    return np.ndim(x) == 0


class _OwnedArray(np.ndarray):
    """A read-only host array that keeps the integrator it was read from
    alive, as the reference's views do (their base object is the integrator:
    heyoka/expose_batch_integrators.cpp:394-541)."""

    def __array_finalize__(self, obj):
        self._owner = getattr(obj, "_owner", None)


def _owned(a, owner):
    # The array under the view is made read-only too, so that the view's
    # writeability cannot be turned back on (as with the reference's arrays).
    base = np.asarray(a)
    base.flags.writeable = False
    v = base.view(_OwnedArray)
    v._owner = owner
    return v


def _callbacks(cb):
    """The step callbacks of a ``callback=`` argument: none, one, or a list
    (a callback set: every one is called after each step)."""
    if cb is None:
        return []
    return list(cb) if isinstance(cb, (list, tuple)) else [cb]


def _run_callbacks(cbs, ta):
    """Call every step callback on the integrator; False if any asks to stop
    (reference: heyoka/step_cb_utils.cpp:65-90, the return value must be a bool)."""
    go = True
    for cb in cbs:
        ret = cb(ta)
        if not isinstance(ret, (bool, np.bool_)):
            raise TypeError(
                "The call operator of a step callback is expected to return a boolean, but a value of type '{}' "
                "was returned instead".format(str(type(ret))))
        go = go and bool(ret)
    return go


def _dev_index(device):
    if device is None:
        if not torch.cuda.is_available():
            raise _lib.HykError("the GPU batch integrator needs a CUDA device; none is available")
        return torch.cuda.current_device()
    d = torch.device(device)
    if d.type != "cuda":
        raise ValueError("the GPU batch integrator runs on CUDA devices only, not '{}'".format(device))
    return d.index if d.index is not None else torch.cuda.current_device()


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _dadd(xh, xl, yh, yl):
    s, e = _two_sum(xh, yh)
    e = e + (xl + yl)
    hi = s + e
    return hi, e - (hi - s)


class LaneArray(torch.Tensor):
    """A device tensor that also accepts what the reference's NumPy views
    accept: assignment from lists, tuples and NumPy arrays (converted to
    the tensor's dtype on its device), comparison with them, and conversion
    with ``numpy.asarray``."""

    def _coerce(self, value):
        if isinstance(value, torch.Tensor):
            return value.to(device=self.device, dtype=self.dtype)
        a = _to_fp_array(value, "value", np.float32 if self.dtype == torch.float32 else np.float64)
        if not a.flags.writeable:  # a read-only view (tstate, d_output, ...): torch wants its own copy
            a = a.copy()
        return torch.as_tensor(a, device=self.device)

    def __setitem__(self, idx, value):
        super().__setitem__(idx, self._coerce(value))

    # Comparisons give host NumPy arrays, as comparisons of the reference's views do.
    def __eq__(self, other):
        return torch.Tensor.__eq__(self.as_subclass(torch.Tensor), self._coerce(other)).cpu().numpy()

    def __ne__(self, other):
        return torch.Tensor.__ne__(self.as_subclass(torch.Tensor), self._coerce(other)).cpu().numpy()

    __hash__ = torch.Tensor.__hash__

    def __array__(self, dtype=None, copy=None):
        a = self.detach().as_subclass(torch.Tensor).cpu().numpy()
        return a if dtype is None else a.astype(dtype)


class taylor_adaptive_batch:
    """Adaptive Taylor integrator over a batch of lanes, one GPU thread per lane."""

    def __init__(
        self,
        sys,
        state,
        time=None,
        pars=None,
        tol=0.0,
        high_accuracy=False,
        compact_mode=False,
        t_events=[],  # noqa: B006 - mirrors the reference signature
        nt_events=[],  # noqa: B006
        parallel_mode=False,
        *,
        fp_type=float,
        device=None,
        prop_mode="persistent",
        block_lanes=0,
        pin_arith=False,
        schedule="lpt",
        team_size=0,
        persist_ctas=0,
        global_jets=False,
        autotune=False,
        batch_semantics="reference",
        cold_rows=True,
        debug=False,
        **kwargs,
    ):
        llvm = {"opt_level": 3, "force_avx512": False, "slp_vectorize": False, "fast_math": False,
                "code_model": code_model.small, "parjit": False}
        for k in list(kwargs):
            if k in _LLVM_KWARGS:
                llvm[k] = kwargs.pop(k)
                warnings.warn(
                    "the LLVM option '{}' has no effect on the GPU batch integrator".format(k), stacklevel=2
                )
        self._llvm = llvm
        if kwargs:
            raise TypeError("unexpected keyword argument(s): {}".format(", ".join(sorted(kwargs))))
        self._np_dt, self._tdt = _fp_of(fp_type)
        f32 = self._tdt == torch.float32
        self._high_accuracy = bool(high_accuracy)
        from .events import nt_event_batch, t_event_batch

        t_events, nt_events = list(t_events), list(nt_events)
        for e in t_events:
            if not isinstance(e, t_event_batch):
                raise TypeError("the t_events argument must be a list of t_event_batch objects")
        for e in nt_events:
            if not isinstance(e, nt_event_batch):
                raise TypeError("the nt_events argument must be a list of nt_event_batch objects")
        self._t_events = _copy.deepcopy(t_events)
        self._nt_events = _copy.deepcopy(nt_events)
        if prop_mode not in _PROP_MODES:
            raise ValueError("prop_mode must be 'persistent', 'plain' or 'plain_inplace'")
        if schedule not in ("lpt", "fifo"):
            raise ValueError("schedule must be 'lpt' or 'fifo'")
        from .var import var_ode_sys

        self._vsys = sys if isinstance(sys, var_ode_sys) else None
        if self._vsys is not None:
            sys = self._vsys.sys

        st = _to_fp_array(state, "state", self._np_dt)
        if st.ndim != 2:
            raise ValueError(
                "Invalid state vector passed to the constructor of a batch integrator: "
                "the expected number of dimensions is 2, but the input array has a dimension of {}".format(st.ndim)
            )
        B = st.shape[1]
        evs = [(e.expression, True, int(e.direction), e.cooldown) for e in self._t_events]
        evs += [(e.expression, False, int(e.direction), -1.0) for e in self._nt_events]
        self._dec = taylor_decompose(sys, events=evs)
        if st.shape[0] == 0:
            st = np.zeros((self._dec.n_eq, B), dtype=self._np_dt)  # an empty initial state means zeros (the reference's rule)
        np_ = self._dec.n_pars
        if pars is not None:
            pa = np.asarray(pars)
            if pa.ndim != 2 or pa.shape[1] != B:
                raise ValueError(
                    "Invalid parameter vector passed to the constructor of a batch integrator: "
                    "the expected array shape is (n, {}), but the input array has either the wrong "
                    "number of dimensions or the wrong shape".format(B)
                )
            pa = _to_fp_array(pa, "pars", self._np_dt)
            if pa.shape[0] < np_:
                raise ValueError(
                    "Invalid number of parameter values passed to the constructor of an adaptive "
                    "Taylor integrator: {} parameter value(s) were passed, but the ODE system contains "
                    "{} parameter(s)".format(pa.shape[0] * B, np_ * B)
                )
        else:
            pa = np.zeros((np_, B), dtype=self._np_dt)
        if time is not None:
            ti = np.asarray(time)
            if ti.ndim != 1 or ti.shape[0] != B:
                raise ValueError(
                    "Invalid time vector passed to the constructor of a batch integrator: "
                    "the expected array shape is ({}), but the input array has either the wrong "
                    "number of dimensions or the wrong shape".format(B)
                )
            ti = _to_fp_array(ti, "time", self._np_dt)
        else:
            ti = np.zeros(B, dtype=self._np_dt)
        if self._vsys is not None and st.shape[0] == self._vsys.n_orig_sv:
            # the variational part starts from the identity (state arguments), zero (parameters)
            # and, for the initial time, values computed from the state, the parameters and t0
            if self._vsys.has_time:
                st = np.concatenate([st, self._vsys.initial_variational_state_at(
                    st, ti, pa[: self._dec.n_pars] if self._dec.n_pars else None).astype(self._np_dt)])
            else:
                st = np.concatenate([st, self._vsys.initial_variational_state(B).astype(self._np_dt)])
        if st.shape[0] != self._dec.n_eq:
            raise ValueError(
                "Inconsistent sizes detected in the initialization of an adaptive Taylor integrator: "
                "the state vector has a dimension of {}, while the number of equations is {}".format(
                    st.shape[0], self._dec.n_eq
                )
            )
        if B == 0:
            raise ValueError("The batch size in an adaptive Taylor integrator cannot be zero")
        tol = float(self._np_dt(tol))
        if tol == 0.0:
            tol = float(np.finfo(self._np_dt).eps)
        self._tol = tol
        self._order = order_from_tol(tol)
        self._dev = _dev_index(device)
        self._tdev = torch.device("cuda", self._dev)
        self._autotune = None
        if autotune and not pin_arith and not (self._t_events or self._nt_events):
            # measured choice of the kernel form and block size (cached per system)
            from .autotune import tune

            r = tune(taylor_decompose(sys), st, pars=pa if np_ else None, tol=tol, fp_type=fp_type,
                     high_accuracy=self._high_accuracy, device=torch.device("cuda", self._dev))
            best = r["best"]
            team_size, global_jets, block_lanes = best["team_size"], best["global_jets"], best["block_lanes"]
            self._autotune = r
        self._mod_opts = dict(block_lanes=int(block_lanes), pin_arith=bool(pin_arith), team_size=int(team_size),
                              persist_ctas=int(persist_ctas), high_accuracy=self._high_accuracy,
                              global_jets=bool(global_jets), float32=f32, cold_rows=bool(cold_rows),
                              debug=bool(debug))
        self._mod = get_module(self._dec, self._order, self._dev, **self._mod_opts)
        # propagate_grid's own measured choice, when the autotuner found a
        # different one (its modules share the bookkeeping layout)
        self._mod_grid_opts = None
        self._mod_grid = None
        bg = self._autotune.get("best_grid") if self._autotune else None
        if bg and (bg["team_size"], bg["global_jets"], bg["block_lanes"]) != (team_size, global_jets, block_lanes):
            self._mod_grid_opts = dict(self._mod_opts, team_size=int(bg["team_size"]),
                                       global_jets=bool(bg["global_jets"]), block_lanes=int(bg["block_lanes"]))
            self._mod_grid = get_module(self._dec, self._order, self._dev, **self._mod_grid_opts)
        self._prop_mode = prop_mode
        self._schedule = schedule
        if batch_semantics not in ("reference", "lane"):
            raise ValueError("batch_semantics must be 'reference' or 'lane', not {!r}".format(batch_semantics))
        self._batch_semantics = batch_semantics
        self._compact_mode = bool(compact_mode)
        self._B = B
        fr = dict(dtype=self._tdt, device=self._tdev)
        self._state = torch.tensor(st, **fr).contiguous()
        self._pars = torch.tensor(pa, **fr).contiguous()
        self._thi = torch.tensor(ti, **fr)
        self._tlo = torch.zeros(B, **fr)
        self._last_h = torch.zeros(B, **fr)
        self._tc = torch.zeros((self._dec.n_eq, self._order + 1, B), **fr)
        self._d_out = torch.zeros((self._dec.n_eq, B), **fr)
        self._step_res = None
        self._prop = None  # dict of device arrays of the last propagation
        self._final_tc_mask = None  # lanes whose tc must be the final-state jets
        self._launch_events = None
        self._ev = self._ev_alloc(16) if (self._t_events or self._nt_events) else None

    # ------------------------------------------------------------------ properties
    @property
    def state(self):
        return self._state.as_subclass(LaneArray)

    @property
    def pars(self):
        return self._pars.as_subclass(LaneArray)

    @property
    def time(self):
        return _owned(self._thi.cpu().numpy(), self)

    @property
    def dtime(self):
        return _owned(self._thi.cpu().numpy(), self), _owned(self._tlo.cpu().numpy(), self)

    @property
    def order(self):
        return self._order

    @property
    def tol(self):
        return self._tol

    @property
    def dim(self):
        return self._dec.n_eq

    @property
    def batch_size(self):
        return self._B

    @property
    def compact_mode(self):
        return self._compact_mode

    @property
    def llvm_state(self):
        return _LLVMStateInfo(self, self.__dict__.get("_llvm", {}))

    @property
    def fp_type(self):
        return float if self._np_dt == np.float64 else np.float32

    @property
    def high_accuracy(self):
        return self._high_accuracy

    @property
    def with_events(self):
        return bool(self._t_events or self._nt_events)

    @property
    def decomposition(self):
        return self._dec.as_list()

    @property
    def sys(self):
        return list(self._dec.sys)

    @property
    def is_variational(self):
        return self._vsys is not None

    @property
    def n_orig_sv(self):
        return self._vsys.n_orig_sv if self._vsys is not None else self.dim

    @property
    def vargs(self):
        return list(self._vsys.vargs) if self._vsys is not None else []

    @property
    def vorder(self):
        return self._vsys.order if self._vsys is not None else 0

    def get_vslice(self, order, component=None):
        if self._vsys is None:
            raise ValueError("The integrator is not variational")
        return self._vsys.vslice(order, component)

    def get_mindex(self, i):
        if self._vsys is None:
            raise ValueError("The integrator is not variational")
        return self._vsys.mindex(i)

    def _tstate_buf(self):
        buf = self.__dict__.get("_tstate")
        if buf is None:
            buf = np.zeros((self.n_orig_sv, self._B), dtype=self._np_dt)
            self._tstate = buf
        return buf

    @property
    def tstate(self):
        """The result of the last ``eval_taylor_map`` (read-only, shape (n_orig_sv, batch_size))."""
        if self._vsys is None:
            raise ValueError("The integrator is not variational")
        return _owned(self._tstate_buf(), self)

    def eval_taylor_map(self, inputs):
        """Evaluate the Taylor map of the variational state at the argument
        displacements ``inputs`` (shape (n_vargs, batch_size)): for every
        original state variable, sum over the multi-indices alpha of
        X_alpha delta^alpha / alpha! (reference:
        heyoka/expose_batch_integrators.cpp:549-649).  Returns ``tstate``."""
        if self._vsys is None:
            raise ValueError("The integrator is not variational")
        m, B = len(self._vsys.vargs), self._B
        if isinstance(inputs, torch.Tensor):
            if inputs.device.type == "cuda" and inputs.untyped_storage().data_ptr() == \
                    self._state.untyped_storage().data_ptr():
                raise ValueError("The array of inputs provided for the evaluation of a Taylor map may overlap "
                                 "with the internal state of the integrator")
            inputs = inputs.detach().cpu().numpy()
        arr = np.asarray(inputs)
        if arr.dtype != self._np_dt:
            if np.issubdtype(arr.dtype, np.integer) and isinstance(inputs, np.ndarray):
                raise TypeError("Invalid dtype detected for the inputs of a Taylor map evaluation: the expected "
                                "dtype is {}, but the dtype is {} instead".format(np.dtype(self._np_dt).name, arr.dtype))
            arr = arr.astype(self._np_dt)
        if isinstance(inputs, np.ndarray) and not inputs.flags.c_contiguous:
            raise ValueError("Invalid inputs array detected in a Taylor map evaluation: the array is not C-style "
                             "contiguous, please consider using numpy.ascontiguousarray() to turn it into one")
        if arr.ndim != 2:
            raise ValueError("The array of inputs provided for the evaluation of a Taylor map has {} dimension(s), "
                             "but it must have 2 dimensions instead".format(arr.ndim))
        if arr.shape[0] != m:
            raise ValueError("The array of inputs provided for the evaluation of a Taylor map has {} row(s), but it "
                             "must have {} row(s) instead".format(arr.shape[0], m))
        if arr.shape[1] != B:
            raise ValueError("The array of inputs provided for the evaluation of a Taylor map has {} column(s), but "
                             "it must have {} column(s) instead".format(arr.shape[1], B))
        buf = self._tstate_buf()
        if np.shares_memory(arr, buf):
            raise ValueError("The array of inputs provided for the evaluation of a Taylor map may overlap with "
                             "the internal state of the integrator")
        st = self._state.cpu().numpy()
        out = np.zeros((self.n_orig_sv, B), dtype=self._np_dt)
        for row, comp, a, inv_fact in self._vsys.taylor_map_terms():
            term = st[row] * self._np_dt(inv_fact)
            for j, e in enumerate(a):
                if e:
                    term = term * arr[j] ** e
            out[comp] += term
        buf.flags.writeable = True  # the buffer owns its memory; the views handed out stay read-only
        buf[...] = out
        buf.flags.writeable = False
        return self.tstate

    @property
    def device(self):
        return self._tdev

    @property
    def module_info(self):
        """Compiled-kernel facts: block size, shared memory per lane, registers, flops per step."""
        return self._mod.info_dict()

    @property
    def prop_mode(self):
        return self._prop_mode

    @prop_mode.setter
    def prop_mode(self, v):
        if v not in _PROP_MODES:
            raise ValueError("prop_mode must be 'persistent', 'plain' or 'plain_inplace'")
        self._prop_mode = v

    @property
    def last_h(self):
        return _owned(self._last_h.cpu().numpy(), self)

    @property
    def tc(self):
        self._refresh_final_tc()
        return _owned(self._tc.cpu().numpy(), self)

    @property
    def d_output(self):
        return _owned(self._d_out.cpu().numpy(), self)

    @property
    def step_res(self):
        if self._step_res is None:
            return [(taylor_outcome.success, 0.0)] * self._B
        oc, h = self._step_res
        oc, h = oc.cpu().numpy(), h.cpu().numpy()
        return [(taylor_outcome(int(o)), float(x)) for o, x in zip(oc, h)]

    @property
    def propagate_res(self):
        if self._prop is None:
            return [(taylor_outcome.success, math.inf, 0.0, 0)] * self._B
        p = self._prop
        oc = p["outcome"].cpu().numpy()
        mn, mx = p["min_h"].cpu().numpy(), p["max_h"].cpu().numpy()
        ns = p["n_steps"].cpu().numpy()
        return [(taylor_outcome(int(a)), float(b), float(c), int(d)) for a, b, c, d in zip(oc, mn, mx, ns)]

    @property
    def te_cooldowns(self):
        """Per lane, per terminal event: None, or (time of the last trigger,
        cooldown) while the event's cooldown applies (reference:
        heyoka/expose_batch_integrators.cpp te_cooldowns)."""
        if self._ev is None:
            return [[] for _ in range(self._B)]
        last = self._ev["last"].cpu().numpy()
        out = []
        for b in range(self._B):
            row = []
            for j, e in enumerate(self._t_events):
                t = float(last[j, b])
                if t != t:
                    row.append(None)
                else:
                    rel = 1e-12 if self._np_dt == np.float64 else float(np.float32(5e-4))
                    cd = e.cooldown if e.cooldown >= 0 else rel * max(1.0, abs(t))
                    row.append((t, cd))
            out.append(row)
        return out

    def reset_cooldowns(self, i=None):
        """Forget the terminal events' cooldowns, of lane ``i`` or of every lane."""
        if self._ev is None:
            return
        if i is None:
            self._ev["last"].fill_(math.nan)
        else:
            i = int(i)
            if not 0 <= i < self._B:
                raise ValueError("Cannot reset the cooldowns at batch index {}: the batch size is only {}".format(
                    i, self._B))
            self._ev["last"][:, i] = math.nan

    @property
    def t_events(self):
        from .events import _BoundEvent

        return [_BoundEvent(self, e) for e in self._t_events]

    @property
    def nt_events(self):
        from .events import _BoundEvent

        return [_BoundEvent(self, e) for e in self._nt_events]

    # ------------------------------------------------------------------ events
    def _ev_alloc(self, cap):
        B, f = self._B, dict(device=self._tdev)
        nt = max(len(self._t_events), 1)
        return {
            "cap": cap,
            "t_hi": torch.empty((cap, B), dtype=self._tdt, **f),
            "t_lo": torch.empty((cap, B), dtype=self._tdt, **f),
            "info": torch.empty((cap, B), dtype=torch.int32, **f),
            "count": torch.zeros(B, dtype=torch.int64, **f),
            "last": torch.full((nt, B), math.nan, dtype=self._tdt, **f),
            "sign": torch.zeros(B, dtype=torch.int32, **f),
        }

    def _ev_grow(self):
        old = self._ev
        new = self._ev_alloc(2 * old["cap"])
        c = old["cap"]
        for k in ("t_hi", "t_lo", "info"):
            new[k][:c] = old[k]
        for k in ("count", "last", "sign"):
            new[k] = old[k]
        self._ev = new

    def _ev_scratch(self):
        """Throw-away event buffers for the internal steps that are not taken
        (estimates): their roots must not reach the integrator's records."""
        if self._ev is None:
            return None
        saved = self._ev
        self._ev = self._ev_alloc(1)
        self._ev["last"] = saved["last"].clone()
        d = self._ev_fill(_lib.hyk_prop_t())
        self._ev_keep = self._ev  # alive until the next internal step
        self._ev = saved
        return d

    def _ev_fill(self, d):
        """Point the event fields of a hyk_prop_t at the integrator's buffers."""
        ev = self._ev
        if ev is None:
            return d
        d.ev_t_hi, d.ev_t_lo, d.ev_info = ev["t_hi"].data_ptr(), ev["t_lo"].data_ptr(), ev["info"].data_ptr()
        d.ev_count, d.ev_capacity = ev["count"].data_ptr(), ev["cap"]
        d.ev_last, d.ev_sign = ev["last"].data_ptr(), ev["sign"].data_ptr()
        return d

    def _ev_target(self, b):
        """The integrator and lane of batch lane b: this one, or in an
        ensemble's combined batch the lane's iteration.  Its callbacks are
        given ``_ev_arg`` of it."""
        route = self.__dict__.get("_ev_route")
        if route is None:
            return self, b
        views, B = route
        return views[b // B], b % B

    @staticmethod
    def _ev_arg(tgt):
        """The integrator an event callback is given: the scalar integrator a
        one-lane batch stands for, when there is one."""
        return tgt.__dict__.get("_scalar") or tgt

    def _ev_dispatch_nt(self):
        """Run the non-terminal callbacks for the recorded roots, in
        chronological order per lane, then empty the records."""
        from .events import callback_error

        ev = self._ev
        cnt = ev["count"].cpu().numpy()
        if not cnt.any():
            return
        K = int(cnt.max())
        hi = ev["t_hi"][:K].cpu().numpy()
        lo = ev["t_lo"][:K].cpu().numpy()
        info = ev["info"][:K].cpu().numpy()
        ev["count"].zero_()
        for b in np.nonzero(cnt)[0]:
            n = int(cnt[b])
            th, tl, inf = hi[:n, b], lo[:n, b], info[:n, b]
            fwd = n < 2 or (th[-1] + tl[-1]) >= (th[0] + tl[0])
            order = np.lexsort((tl, th)) if fwd else np.lexsort((-tl, -th))
            tgt, lb = self._ev_target(int(b))
            for r in order:
                k, sg = int(inf[r]) >> 2, (int(inf[r]) & 3) - 1
                cb = tgt._nt_events[k].callback
                try:
                    cb(self._ev_arg(tgt), float(th[r]), sg, lb)
                except Exception as exc:  # noqa: BLE001 - re-raised as the reference does
                    raise callback_error(exc) from exc

    def _ev_terminal(self, lanes_oc):
        """Terminal callbacks for the lanes a terminal event stopped
        (lanes_oc: {lane: event index}); returns the lanes whose callback
        asked to continue."""
        from .events import callback_error, check_bool_retval

        if not lanes_oc:
            return []
        sg = self._ev["sign"].cpu().numpy()
        resume = []
        for b, k in sorted(lanes_oc.items()):
            tgt, lb = self._ev_target(int(b))
            cb = tgt._t_events[k].callback
            if cb is None:
                continue
            try:
                ret = cb(self._ev_arg(tgt), int(sg[b]), lb)
            except Exception as exc:  # noqa: BLE001
                raise callback_error(exc) from exc
            if check_bool_retval(ret):
                resume.append(b)
        return resume

    @property
    def propagate_res_tensors(self):
        """Device tensors of the last propagation: outcome, min_h, max_h, n_steps, n_iter."""
        if self._prop is None:
            return None
        return {k: self._prop[k] for k in ("outcome", "min_h", "max_h", "n_steps", "n_iter")}

    # ------------------------------------------------------------------ time
    def _lane_vec(self, v, what):
        if _is_scalar(v):
            return torch.full((self._B,), float(self._np_dt(v)), dtype=self._tdt, device=self._tdev)
        a = _to_fp_array(v, what, self._np_dt)
        if a.ndim != 1 or a.shape[0] != self._B:
            raise ValueError(
                "Invalid {} passed to a batch integrator: the expected array shape is ({}), "
                "but the input array has either the wrong number of dimensions or the wrong shape".format(
                    what, self._B
                )
            )
        return torch.tensor(a, dtype=self._tdt, device=self._tdev)

    def set_time(self, time):
        t = self._lane_vec(time, "time vector")
        self._thi.copy_(t)
        self._tlo.zero_()

    def set_dtime(self, hi_time, lo_time):
        if _is_scalar(hi_time) != _is_scalar(lo_time):
            raise TypeError("The two arguments to the set_dtime() method must be of the same type")
        hi = self._lane_vec(hi_time, "time vector")
        lo = self._lane_vec(lo_time, "time vector")
        if not (torch.isfinite(hi).all() and torch.isfinite(lo).all()):
            raise ValueError("Non-finite time values passed to set_dtime()")
        s, e = _two_sum(hi, lo)
        self._thi.copy_(s)
        self._tlo.copy_(e)

    # ------------------------------------------------------------------ stepping
    def _step(self, max_delta_t, backward, write_tc):
        L = _lib.load()
        B = self._B
        oc = torch.empty(B, dtype=torch.int64, device=self._tdev)
        h = torch.empty(B, dtype=self._tdt, device=self._tdev)
        md = None
        if max_delta_t is not None:
            md = self._lane_vec(max_delta_t, "max_delta_t vector")
            if torch.isnan(md).any():
                raise ValueError("A NaN max_delta_t was passed to the step() function of an adaptive Taylor integrator")
        lanes = lanes_struct(self._state, self._pars, self._thi, self._tlo)
        evd = None
        if self._ev is not None:
            while self._ev["cap"] < 64:  # room for the roots of one step (records are emptied after each call)
                self._ev_grow()
            evd = self._ev_fill(_lib.hyk_prop_t())
        with torch.cuda.device(self._dev):
            _lib.check(
                L.hyk_step(
                    self._mod.handle, lanes, None if md is None else md.data_ptr(), int(backward),
                    oc.data_ptr(), h.data_ptr(), self._tc.data_ptr() if write_tc else None, evd,
                    stream_handle(self._dev),
                ),
                "hyk_step",
            )
        self._step_res = (oc, h)
        self._last_h = h.clone()
        if write_tc:
            self._final_tc_mask = None
        if self._ev is not None:
            ocn = oc.cpu().numpy()
            if (ocn == _lib.OC_EV_OVERFLOW).any():
                raise RuntimeError("a step found more event roots than the event buffers hold")
            self._ev_dispatch_nt()
            self._ev_terminal({int(b): int(o) for b, o in enumerate(ocn) if o >= 0})

    def step(self, max_delta_t=None, write_tc=False):
        """One step on every lane (optionally clamped by a per-lane ``max_delta_t``)."""
        if isinstance(max_delta_t, bool):
            write_tc, max_delta_t = max_delta_t, None
        if max_delta_t is not None and _is_scalar(max_delta_t):
            raise TypeError("the max_delta_t argument of the batch step() function must be a vector")
        self._step(max_delta_t, False, write_tc)

    def step_backward(self, write_tc=False):
        self._step(None, True, write_tc)

    # ------------------------------------------------------------------ dense output
    def update_d_output(self, t, rel_time=False):
        self._refresh_final_tc()
        tt = self._lane_vec(t, "time vector")
        if rel_time:
            dt = self._last_h + tt
        else:
            # (t - (time - last_h)) in double-length arithmetic.
            sh, sl = _dadd(self._thi, self._tlo, -self._last_h, torch.zeros_like(self._last_h))
            dt, _ = _dadd(tt, torch.zeros_like(tt), -sh, -sl)
        L = _lib.load()
        fn = L.hyk_dense_eval_f32 if self._tdt == torch.float32 else L.hyk_dense_eval
        with torch.cuda.device(self._dev):
            _lib.check(
                fn(
                    self._tc.data_ptr(), self.dim, self._order, self._B, self._B, dt.contiguous().data_ptr(),
                    self._d_out.data_ptr(), stream_handle(self._dev),
                ),
                "hyk_dense_eval",
            )
        return self.d_output

    def _refresh_final_tc(self):
        """Lanes that finished before the batch's last iteration: the reference's
        tc holds the jets of their final state (computed by its zero steps)."""
        mask = self._final_tc_mask
        if mask is None:
            return
        self._final_tc_mask = None
        if not bool(mask.any()):
            return
        tc = torch.empty_like(self._tc)
        st, th, tl = self._state.clone(), self._thi.clone(), self._tlo.clone()
        zero = torch.zeros(self._B, dtype=self._tdt, device=self._tdev)
        oc = torch.empty(self._B, dtype=torch.int64, device=self._tdev)
        h = torch.empty_like(zero)
        L = _lib.load()
        with torch.cuda.device(self._dev):
            _lib.check(
                L.hyk_step(
                    self._mod.handle, lanes_struct(st, self._pars, th, tl), zero.data_ptr(), 0, oc.data_ptr(),
                    h.data_ptr(), tc.data_ptr(), self._ev_scratch(), stream_handle(self._dev),
                ),
                "hyk_step",
            )
        self._tc = torch.where(mask.view(1, 1, -1), tc, self._tc)

    # ------------------------------------------------------------------ propagation
    def _check_prop_args(self, max_delta_t, callback):
        for cb in _callbacks(callback):
            if not callable(cb):
                raise TypeError(
                    "An object of type '{}' cannot be used as a step callback because it is not callable".format(
                        str(type(cb))))
        if max_delta_t is None or (not _is_scalar(max_delta_t) and len(max_delta_t) == 0):
            return None
        md = self._lane_vec(max_delta_t, "max_delta_t vector")
        if torch.isnan(md).any():
            raise ValueError("A nan max_delta_t was passed to the propagate_*() functions of an adaptive Taylor integrator")
        if (md <= 0).any():
            raise ValueError(
                "A non-positive max_delta_t was passed to the propagate_*() functions of an adaptive Taylor integrator"
            )
        return md

    def _alloc_prop(self, with_grid):
        B, f = self._B, dict(device=self._tdev)
        p = {
            "rem_hi": torch.empty(B, dtype=self._tdt, **f),
            "rem_lo": torch.empty(B, dtype=self._tdt, **f),
            "outcome": torch.empty(B, dtype=torch.int64, **f),
            "min_h": torch.empty(B, dtype=self._tdt, **f),
            "max_h": torch.empty(B, dtype=self._tdt, **f),
            "n_steps": torch.empty(B, dtype=torch.int64, **f),
            "n_iter": torch.empty(B, dtype=torch.int64, **f),
            "grid_idx": torch.empty(B, dtype=torch.int64, **f) if with_grid else None,
            "last_h": torch.empty(B, dtype=self._tdt, **f),
            "status": torch.empty(B, dtype=torch.int32, **f),
        }
        return p

    def _ev_has_callbacks(self):
        return bool(self._nt_events) or any(e.callback is not None for e in self._t_events)

    def _run(self, tf_hi, tf_lo, max_steps, md, grid=None, write_tc=False, c_output=False, group=None,
             lane_order=None, callback=None, group_callbacks=None):
        """A propagation of every lane to (tf_hi, tf_lo), with the batch rules
        of ``batch_semantics``.

        "reference" (the default): a state that becomes non-finite stops every
        lane of its batch (of its ensemble iteration, with ``group``) at that
        iteration, with err_nf_state for the lane concerned and the outcome of
        its last step for the others, as the reference's batch propagate loop
        does (heyoka/expose_batch_integrators.cpp:279-314); event callbacks run
        after each batch step.  The one-launch-per-step and the stepped forms
        step the lanes in lockstep, so the stop is exact in one pass; the
        persistent form lets lanes run ahead, so after a pass in which a
        state became non-finite the initial state is restored and the
        propagation runs again with every lane stopping at the iteration the
        first pass found.  "lane": a non-finite state stops only its lane, and
        event callbacks run when the propagation returns."""
        ref = self.__dict__.get("_batch_semantics", "reference") == "reference"
        stepped_ev = ref and self._ev is not None and self._ev_has_callbacks()
        if not ref:
            return self._run_once(tf_hi, tf_lo, max_steps, md, grid, write_tc, c_output, group, lane_order, callback,
                                  group_callbacks, None, False)
        B = self._B
        G = B if group is None else int(group)
        stop = torch.full((B // G,), -1, dtype=torch.int64, device=self._tdev)  # all ones: no stop
        if stepped_ev or bool(_callbacks(callback)) or bool(group_callbacks):
            # one batch step per launch: a launch in which a state became
            # non-finite is taken again with the stop words it left (_run_once)
            return self._run_once(tf_hi, tf_lo, max_steps, md, grid, write_tc, c_output, group, lane_order, callback,
                                  group_callbacks, (stop, G), stepped_ev)
        snap = (self._state.clone(), self._thi.clone(), self._tlo.clone(),
                None if self._ev is None else {k: self._ev[k].clone() for k in ("count", "last", "sign")})
        res = self._run_once(tf_hi, tf_lo, max_steps, md, grid, write_tc, c_output, group, lane_order, callback,
                             group_callbacks, (stop, G), False)
        if bool((stop != -1).any()):
            # a state became non-finite: run again from the initial state, every
            # lane of the group taking the failing iteration uncounted and stopping
            self._state.copy_(snap[0])
            self._thi.copy_(snap[1])
            self._tlo.copy_(snap[2])
            if snap[3] is not None:
                for k, v in snap[3].items():
                    self._ev[k].copy_(v)
            res = self._run_once(tf_hi, tf_lo, max_steps, md, grid, write_tc, c_output, group, lane_order, callback,
                                 group_callbacks, (stop, G), False)
        return res

    def _run_once(self, tf_hi, tf_lo, max_steps, md, grid, write_tc, c_output, group, lane_order, callback,
                  group_callbacks, stop, stepped_ev):
        """Initialise and run a propagation of every lane to (tf_hi, tf_lo).

        With step callbacks the persistent kernel runs one step per lane per
        launch (its bookkeeping is resumable), and the callbacks are called on
        the host after each such batch step; one returning False stops every
        lane with the ``cb_stop`` outcome (reference:
        heyoka/expose_batch_integrators.cpp:243-392, callback semantics in
        heyoka/step_cb_utils.cpp:65-112).

        ``group_callbacks`` (ensembles): one ``(integrator, callbacks)`` per
        group of ``group`` lanes, called after each batch step in which the
        group stepped; False stops that group's lanes only."""
        L = _lib.load()
        cbs = _callbacks(callback)
        for cb in cbs:
            if hasattr(cb, "pre_hook"):
                cb.pre_hook(self)
        gcbs = group_callbacks or []
        for view, cl in gcbs:
            for cb in cl:
                if hasattr(cb, "pre_hook"):
                    cb.pre_hook(view)
        stepped = cbs or gcbs or stepped_ev  # one batch step per launch
        if max_steps < 0:
            raise ValueError("max_steps must be non-negative")
        B, ne, order = self._B, self.dim, self._order
        p = self._alloc_prop(grid is not None)
        grid_out = None
        if grid is not None:
            grid_out = torch.empty((grid.shape[0], ne, B), dtype=self._tdt, device=self._tdev)
        want_tc = write_tc or c_output
        last_tc = torch.empty_like(self._tc) if want_tc else None
        cap = 0
        tcs = thi = tlo = None
        if c_output:
            cap = 64
            tcs = torch.empty((cap, ne, order + 1, B), dtype=self._tdt, device=self._tdev)
            thi = torch.empty((cap, B), dtype=self._tdt, device=self._tdev)
            tlo = torch.empty((cap, B), dtype=self._tdt, device=self._tdev)
        t0h, t0l = self._thi.clone(), self._tlo.clone()

        def desc():
            return self._ev_fill(_lib.hyk_prop_t(
                tf_hi.data_ptr(), None if tf_lo is None else tf_lo.data_ptr(), None if md is None else md.data_ptr(),
                int(max_steps),
                None if grid is None else grid.data_ptr(), 0 if grid is None else grid.shape[0],
                None if grid_out is None else grid_out.data_ptr(),
                None if tcs is None else tcs.data_ptr(), None if thi is None else thi.data_ptr(),
                None if tlo is None else tlo.data_ptr(), cap,
                p["rem_hi"].data_ptr(), p["rem_lo"].data_ptr(), p["outcome"].data_ptr(), p["min_h"].data_ptr(),
                p["max_h"].data_ptr(), p["n_steps"].data_ptr(), p["n_iter"].data_ptr(),
                None if p["grid_idx"] is None else p["grid_idx"].data_ptr(), p["last_h"].data_ptr(),
                None if last_tc is None else last_tc.data_ptr(), p["status"].data_ptr(),
                None if lane_order is None else lane_order.data_ptr(),
                0 if lane_order is None else lane_order.numel(), None, None, None, 0, 1 if stepped else 0,
                None, None, None, None, 0, None, None,
                None if stop is None else stop[0].data_ptr(), 0 if stop is None or stop[1] == B else stop[1],
            ))

        lanes = lanes_struct(self._state, self._pars, self._thi, self._tlo)
        mode = _lib.HYK_MODE_PERSISTENT if (self._prop_mode == "persistent" or stepped) else _lib.HYK_MODE_PLAIN
        if lane_order is None and mode == _lib.HYK_MODE_PERSISTENT and self._schedule == "lpt" and B >= 4096:
            lane_order = self._lpt_order(tf_hi, tf_lo)
        done_mask = _lib.LANE_DONE | _lib.LANE_STOPPED
        g_open = None
        if gcbs:
            G = B // len(gcbs)
            g_open = [True] * len(gcbs)  # groups with lanes left to step
        with torch.cuda.device(self._dev):
            s = stream_handle(self._dev)
            d = desc()
            mod = self._mod_grid if (grid is not None and self.__dict__.get("_mod_grid") is not None) else self._mod
            _lib.check(L.hyk_prop_init(mod.handle, lanes, d, s), "hyk_prop_init")
            ev = self._launch_events  # optional (start, end) CUDA events around the propagation launch(es)
            if ev is not None:
                ev[0].record(torch.cuda.current_stream(self._dev))
            ws, ws_bytes = mod.ws, mod.ws_bytes
            if mode == _lib.HYK_MODE_PLAIN and self._prop_mode == "plain":
                # counters plus the list of unfinished lanes the plain form steps
                # (with the counters alone, "plain_inplace", every launch covers
                # every lane)
                ws_bytes = int(L.hyk_propagate_workspace_size(mod.handle, B, mode))
                ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self._tdev)
            while True:
                redo = None
                if stop is not None and stepped:
                    # the step's inputs, to take it again if a state becomes non-finite in it
                    redo = (stop[0].clone(), self._state.clone(), self._thi.clone(), self._tlo.clone(),
                            {k: v.clone() for k, v in p.items() if v is not None},
                            None if self._ev is None else {k: self._ev[k].clone() for k in ("count", "last", "sign")})
                _lib.check(
                    L.hyk_propagate(mod.handle, lanes, d, mode, ws.data_ptr(), ws_bytes, 16, None, s),
                    "hyk_propagate",
                )
                if redo is not None and bool((stop[0] != redo[0]).any()):
                    self._state.copy_(redo[1])
                    self._thi.copy_(redo[2])
                    self._tlo.copy_(redo[3])
                    for k, v in redo[4].items():
                        p[k].copy_(v)
                    if redo[5] is not None:
                        for k, v in redo[5].items():
                            self._ev[k].copy_(v)
                    _lib.check(
                        L.hyk_propagate(mod.handle, lanes, d, mode, ws.data_ptr(), ws_bytes, 16, None, s),
                        "hyk_propagate",
                    )
                if ev is not None:
                    ev[1].record(torch.cuda.current_stream(self._dev))
                if not c_output and self._ev is None and not stepped:
                    break
                full = (p["status"] & _lib.LANE_CAPACITY) != 0
                grow = bool(full.any())
                resume = []
                if self._ev is not None:
                    self._ev_dispatch_nt()
                    evl = (p["status"] & _lib.LANE_EVENT) != 0
                    if bool(evl.any()):
                        idx = torch.nonzero(evl).flatten().cpu().numpy()
                        ks = p["outcome"][evl].cpu().numpy()
                        resume = self._ev_terminal({int(b): -int(k) - 1 for b, k in zip(idx, ks)})
                if stepped:
                    # one batch step done: the callbacks, then the next step
                    # unless every lane is finished
                    finished = (p["status"] & done_mask) != 0
                    settled = bool((finished & ~full).all()) and not resume
                    if gcbs:
                        fin_g = finished.view(len(gcbs), G).all(dim=1).cpu().numpy()
                        for g, (view, cl) in enumerate(gcbs):
                            if not g_open[g]:
                                continue
                            g_open[g] = not fin_g[g]
                            if not _run_callbacks(cl, view) and not fin_g[g]:
                                sl = slice(g * G, (g + 1) * G)
                                p["status"][sl] |= _lib.LANE_STOPPED
                                p["outcome"][sl] = int(taylor_outcome.cb_stop)
                                g_open[g] = False
                        finished = (p["status"] & done_mask) != 0
                        settled = bool((finished & ~full).all()) and not resume
                    if cbs and not _run_callbacks(cbs, self) and not settled:
                        p["outcome"].fill_(int(taylor_outcome.cb_stop))
                        break
                    if settled:
                        break
                elif not grow and not resume:
                    break
                if grow and c_output and bool((p["n_iter"] >= cap).any()):
                    # Grow the coefficient store.
                    ncap = cap * 2
                    ntcs = torch.empty((ncap, ne, order + 1, B), dtype=self._tdt, device=self._tdev)
                    nthi = torch.empty((ncap, B), dtype=self._tdt, device=self._tdev)
                    ntlo = torch.empty((ncap, B), dtype=self._tdt, device=self._tdev)
                    ntcs[:cap] = tcs
                    nthi[:cap] = thi
                    ntlo[:cap] = tlo
                    tcs, thi, tlo, cap = ntcs, nthi, ntlo, ncap
                if grow and self._ev is not None:
                    self._ev_grow()
                # Resume the lanes that filled a store or whose terminal callback said so.
                clear = full
                if resume:
                    r = torch.zeros(B, dtype=torch.bool, device=self._tdev)
                    r[torch.tensor(resume, device=self._tdev)] = True
                    clear = clear | r
                keep = torch.tensor(~(_lib.LANE_CAPACITY | _lib.LANE_STOPPED | _lib.LANE_EVENT), dtype=torch.int32)
                p["status"] = torch.where(clear, p["status"] & keep.to(self._tdev), p["status"])
                d = desc()
        self._finish_prop(p, group, last_tc)
        # Each lane's steps per unit of time over this propagation: the next
        # longest-first queue's estimate of its work (orbits whose step size
        # varies along the orbit are poorly predicted by one step size).
        span = ((self._thi.double() - t0h.double()) + (self._tlo.double() - t0l.double())).abs()
        self._step_rate = torch.where(span > 0, p["n_steps"].double() / span, torch.zeros_like(span))
        res = {"grid_out": grid_out}
        if c_output:
            nrec = p["n_iter"]
            if stop is not None and bool((stop[0] != -1).any()):
                # the lanes stopped at their group's failing iteration took it uncounted
                hit = (stop[0] != -1).repeat_interleave(stop[1])
                unc = hit & ((p["status"] & _lib.LANE_STOPPED) != 0) & (p["outcome"] != int(taylor_outcome.err_nf_state))
                nrec = torch.where(unc | (hit & (p["outcome"] == int(taylor_outcome.err_nf_state))), nrec - 1, nrec)
            res["c_output"] = self._make_c_output(p, tcs, thi, tlo, t0h, t0l, nrec)
        return res

    def _lpt_order(self, tf_hi, tf_lo):
        """Longest-first queue order for the persistent kernel: lanes sorted by
        the estimated number of steps, the lane's measured steps per unit of
        time over its previous propagation times |t_final - t|, or, for a lane
        without one, |t_final - t| / h, h the size of a step from the current
        state (one extra step evaluation, not applied).  The order changes
        only the schedule, never a lane's arithmetic."""
        L = _lib.load()
        B = self._B
        st, th, tl = self._state.clone(), self._thi.clone(), self._tlo.clone()
        oc = torch.empty(B, dtype=torch.int64, device=self._tdev)
        h = torch.empty(B, dtype=self._tdt, device=self._tdev)
        with torch.cuda.device(self._dev):
            _lib.check(
                L.hyk_step(self._mod.handle, lanes_struct(st, self._pars, th, tl), None, 0, oc.data_ptr(),
                           h.data_ptr(), None, self._ev_scratch(), stream_handle(self._dev)),
                "hyk_step",
            )
        rem = (tf_hi.double() - self._thi.double()).abs()
        if tf_lo is not None:
            rem = (rem + tf_lo.double().abs())
        est = torch.nan_to_num(rem / h.double().abs(), nan=0.0, posinf=1e300)
        rate = self.__dict__.get("_step_rate")
        if rate is not None and rate.numel() == B and rate.device == est.device:
            # lanes with a previous propagation: its measured step rate
            est = torch.where(rate > 0, rate * rem, est)
        return torch.argsort(est, descending=True).contiguous()

    def _finish_prop(self, p, group, last_tc):
        """Apply the whole-batch rules that couple the lanes of a batch."""
        B = self._B
        G = B if group is None else group
        ng = B // G
        oc = p["outcome"].view(ng, G)
        hit = (oc == int(taylor_outcome.step_limit)).any(dim=1, keepdim=True)
        oc.copy_(torch.where(hit, torch.full_like(oc, int(taylor_outcome.step_limit)), oc))
        nit = p["n_iter"].view(ng, G)
        gmax = nit.max(dim=1, keepdim=True).values
        early = (nit < gmax).view(B)
        self._last_h = torch.where(early, torch.zeros_like(p["last_h"]), p["last_h"])
        if last_tc is not None:
            self._tc = last_tc
            self._final_tc_mask = early | (p["n_iter"] == 0)
        self._prop = p

    def _make_c_output(self, p, tcs, thi, tlo, t0h, t0l, nrec=None):
        from .c_output import continuous_output_batch

        B = self._B
        nit = p["n_iter"] if nrec is None else nrec
        K = int(nit.max().item()) if B else 0
        ne, order = self.dim, self._order
        fr = dict(dtype=self._tdt, device=self._tdev)
        out_tcs = torch.empty((K, ne, order + 1, B), **fr)
        out_thi = torch.empty((K + 1, B), **fr)
        out_tlo = torch.empty((K + 1, B), **fr)
        out_thi[0], out_tlo[0] = t0h, t0l
        if K:
            out_tcs.copy_(tcs[:K])
            out_thi[1:].copy_(thi[:K])
            out_tlo[1:].copy_(tlo[:K])
            # Zero steps of lanes that finished early: final-state jets, final time.
            self._final_tc_mask = (nit < K) | (nit == 0)
            self._refresh_final_tc()
            idx = torch.arange(K, device=self._tdev).view(K, 1)
            pad = idx >= nit.view(1, B)
            out_tcs = torch.where(pad.view(K, 1, 1, B), self._tc.unsqueeze(0), out_tcs)
            out_thi[1:] = torch.where(pad, self._thi.view(1, B), out_thi[1:])
            out_tlo[1:] = torch.where(pad, self._tlo.view(1, B), out_tlo[1:])
        return continuous_output_batch(out_tcs, out_thi, out_tlo, order, nit.clone())

    def _check_time(self, t, what):
        tt = self._lane_vec(t, what)
        if not bool(torch.isfinite(tt).all()):
            raise ValueError(
                "A non-finite time was passed to the propagate_until() function of an adaptive Taylor integrator"
            )
        return tt

    def propagate_until(self, t, max_steps=0, max_delta_t=[], callback=None, write_tc=False, c_output=False):  # noqa: B006
        """Propagate every lane up to its final time ``t`` (scalar or per lane).

        Returns ``(c_output or None, None)``; per-lane results in ``propagate_res``
        (reference: heyoka/expose_batch_integrators.cpp:279-314)."""
        md = self._check_prop_args(max_delta_t, callback)
        tf = self._check_time(t, "final time vector")
        r = self._run(tf, None, max_steps, md, write_tc=write_tc, c_output=c_output, callback=callback)
        return (r.get("c_output"), callback)

    def propagate_for(self, delta_t, max_steps=0, max_delta_t=[], callback=None, write_tc=False, c_output=False):  # noqa: B006
        """Propagate every lane for ``delta_t`` (scalar or per lane); final time =
        current time + delta_t in double-length arithmetic
        (reference: heyoka/expose_batch_integrators.cpp:243-278)."""
        md = self._check_prop_args(max_delta_t, callback)
        dt = self._check_time(delta_t, "time interval vector")
        hi, lo = _dadd(self._thi, self._tlo, dt, torch.zeros_like(dt))
        r = self._run(hi, lo, max_steps, md, write_tc=write_tc, c_output=c_output, callback=callback)
        return (r.get("c_output"), callback)

    def propagate_grid(self, grid, max_steps=0, max_delta_t=[], callback=None):  # noqa: B006
        """Propagate over a per-lane time grid of shape ``(n, batch_size)``;
        returns ``(None, out)`` with ``out`` of shape ``(n, dim, batch_size)``
        (reference: heyoka/expose_batch_integrators.cpp:315-392)."""
        return (callback, self.propagate_grid_tensor(grid, max_steps, max_delta_t, callback).cpu().numpy())

    def propagate_grid_tensor(self, grid, max_steps=0, max_delta_t=[], callback=None):  # noqa: B006
        """``propagate_grid`` with the output left on the device: a CUDA
        tensor of the integrator's dtype, shape ``(n, dim, batch_size)``."""
        md = self._check_prop_args(max_delta_t, callback)
        g = np.asarray(grid) if not isinstance(grid, torch.Tensor) else grid
        if g.ndim != 2:
            raise ValueError(
                "Invalid grid passed to the propagate_grid() method of a batch integrator: "
                "the expected number of dimensions is 2, but the input array has a dimension of {}".format(g.ndim)
            )
        if g.shape[1] != self._B:
            raise ValueError(
                "Invalid grid passed to the propagate_grid() method of a batch integrator: "
                "the shape must be ({}, {}) but the number of columns is {} instead".format("n", self._B, g.shape[1])
            )
        if isinstance(g, torch.Tensor):
            gd = g.to(device=self._tdev, dtype=self._tdt).contiguous()
        else:
            gd = torch.tensor(_to_fp_array(g, "grid", self._np_dt), dtype=self._tdt, device=self._tdev)
        if gd.shape[0] == 0:
            raise ValueError("Cannot invoke propagate_grid() in a batch integrator if the time grid is empty")
        if not bool(torch.isfinite(gd).all()):
            raise ValueError("A non-finite time value was passed to propagate_grid() in an adaptive Taylor integrator")
        if not bool(((gd[0] == self._thi) & (self._tlo == 0)).all() | (gd[0] == self._thi).all()):
            raise ValueError(
                "When invoking propagate_grid(), the first element of the time grid "
                "must match the current time coordinate"
            )
        if gd.shape[0] > 1:
            dg = gd[1:] - gd[:-1]
            fwd = (dg > 0).all(dim=0)
            bwd = (dg < 0).all(dim=0)
            if not bool((fwd | bwd).all()):
                raise ValueError("A non-monotonic time grid was passed to propagate_grid()")
        tf = gd[-1].contiguous()
        r = self._run(tf, None, max_steps, md, grid=gd, callback=callback)
        return r["grid_out"]

    # ------------------------------------------------------------------ copies
    def __copy__(self):
        return self._clone(deep=False)

    def __deepcopy__(self, memo):
        return self._clone(deep=True, memo=memo)

    def _clone(self, deep, memo=None):
        new = object.__new__(type(self))
        for k, v in self.__dict__.items():
            if isinstance(v, torch.Tensor):
                new.__dict__[k] = v.clone()
            elif k in ("_mod", "_mod_grid", "_dec"):
                new.__dict__[k] = v
            elif k in ("_prop",):
                new.__dict__[k] = None if v is None else {a: (None if b is None else b.clone()) for a, b in v.items()}
            elif k == "_step_res":
                new.__dict__[k] = None if v is None else (v[0].clone(), v[1].clone())
            elif k == "_ev":
                new.__dict__[k] = None if v is None else {a: (b.clone() if isinstance(b, torch.Tensor) else b)
                                                          for a, b in v.items()}
            elif k in ("_t_events", "_nt_events"):
                # a copy of the integrator copies its events (the reference's
                # deep copy gives new callback objects)
                new.__dict__[k] = _copy.deepcopy(v, memo) if deep else list(v)
            elif deep and not k.startswith("_"):
                new.__dict__[k] = _copy.deepcopy(v, memo)
            else:
                new.__dict__[k] = v
        return new

    def debug_record(self, clear=False):
        """With ``debug=True`` (a debug build of the kernels: lane indices
        checked, non-finite Taylor coefficients recorded, nothing trapped):
        ``{"codes": [...], "count": n, "first": {...}}`` of the findings since
        the last clear, the first with its lane, variable, order and
        iteration."""
        if not self._mod_opts.get("debug"):
            raise ValueError("debug_record() needs an integrator constructed with debug=True")
        return self._mod.debug_record(clear)

    def _replica(self, device):
        """A copy of the integrator on another GPU, with that GPU's module (the
        multi-GPU ensemble's per-device template)."""
        d = self.__getstate__()
        d.pop("_scalar", None)
        d["_dev"] = _dev_index(device)
        new = object.__new__(type(self))
        new.__setstate__(d)
        return new

    def __getstate__(self):
        d = {}
        for k, v in self.__dict__.items():
            if k in ("_mod", "_mod_grid"):
                continue
            if isinstance(v, torch.Tensor):
                d[k] = v.cpu()
            elif k == "_prop":
                d[k] = None if v is None else {a: (None if b is None else b.cpu()) for a, b in v.items()}
            elif k == "_step_res":
                d[k] = None if v is None else (v[0].cpu(), v[1].cpu())
            elif k == "_ev":
                d[k] = None if v is None else {a: (b.cpu() if isinstance(b, torch.Tensor) else b) for a, b in v.items()}
            elif k == "_ev_keep":
                continue
            else:
                d[k] = v
        return d

    def __setstate__(self, d):
        dev = torch.device("cuda", d["_dev"]) if torch.cuda.is_available() else None
        self.__dict__.update(d)
        if dev is None:
            raise _lib.HykError("unpickling a GPU batch integrator needs a CUDA device")
        for k, v in list(self.__dict__.items()):
            if isinstance(v, torch.Tensor):
                self.__dict__[k] = v.to(dev)
        if self._prop is not None:
            self._prop = {a: (None if b is None else b.to(dev)) for a, b in self._prop.items()}
        if self._step_res is not None:
            self._step_res = (self._step_res[0].to(dev), self._step_res[1].to(dev))
        if self.__dict__.get("_ev") is not None:
            self._ev = {a: (b.to(dev) if isinstance(b, torch.Tensor) else b) for a, b in self._ev.items()}
        self.__dict__.setdefault("_ev", None)
        self.__dict__.setdefault("_t_events", [])
        self.__dict__.setdefault("_nt_events", [])
        self._tdev = dev
        opts = self.__dict__.get("_mod_opts") or dict(high_accuracy=self.__dict__.get("_high_accuracy", False))
        self._mod = get_module(self._dec, self._order, self._dev, **opts)
        gopts = self.__dict__.get("_mod_grid_opts")
        self._mod_grid = None if gopts is None else get_module(self._dec, self._order, self._dev, **gopts)

    def __repr__(self):
        return (
            "C++ datatype            : {} (GPU, {})\n"
            "Tolerance               : {!r}\n"
            "High accuracy           : false\n"
            "Compact mode            : {}\n"
            "Taylor order            : {}\n"
            "Dimension               : {}\n"
            "Batch size              : {}\n"
            "Time                    : {}\n"
            "State                   : {}\n"
        ).format(
            "double" if self._tdt == torch.float64 else "float", self._tdev, self._tol, str(self._compact_mode).lower(), self._order, self.dim, self._B,
            self.time.tolist() if self._B <= 8 else "[...]",
            self._state.cpu().numpy().tolist() if self._B <= 8 else "[...]",
        )
