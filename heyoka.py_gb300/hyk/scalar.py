"""``taylor_adaptive``: the reference's scalar integrator, as one lane.

The reference's scalar integrator (heyoka/taylor_expose_integrator.cpp:90-420)
integrates one trajectory; its ensembles (``ensemble_propagate_until`` etc.
with a scalar template, heyoka/_ensemble_impl.py:21-68) are the most common
way to integrate many.  Here a scalar integrator is a batch integrator of one
lane with the scalar API on top: 1-D ``state`` and ``pars`` (writable views of
the lane), a float ``time`` and ``dtime`` that can be assigned, ``step``
returning ``(outcome, h)``, ``propagate_until/for`` returning ``(outcome,
min_h, max_h, n_steps, c_output, callback)`` and ``propagate_grid`` returning
``(outcome, min_h, max_h, n_steps, callback, states)``.  Its ensembles run as
one device batch of all the iterations' lanes (``hyk/ensemble.py``).  Its
events (``t_event``/``nt_event``, callbacks without the lane index) run as the
one-lane batch's events, their callbacks called with the scalar integrator.
"""

from __future__ import annotations

import copy as _copy

import numpy as np
import torch

from .integrator import _callbacks, _fp_of, _owned, taylor_adaptive_batch, taylor_outcome


class continuous_output:
    """Dense output of a scalar propagation (reference:
    heyoka/taylor_expose_c_output.cpp:21-258): ``c(t)`` gives the state at t
    (shape (dim,)), ``c(array of n times)`` the states (shape (n, dim)).  The
    host arrays it returns are read-only and keep it alive, as the
    reference's do."""

    def __init__(self, batch_c=None):
        from .c_output import continuous_output_batch

        self._c = continuous_output_batch() if batch_c is None else batch_c

    def _check(self):
        if self._c._tcs is None:
            raise ValueError("Cannot use a default-constructed continuous_output object")

    @property
    def llvm_state(self):
        return self._c.llvm_state

    def __call__(self, t=None, time=None):
        a = np.asarray(t if t is not None else time)
        if a.ndim == 1 and a.size == 0:
            # no times: an empty (0, dim) array, dim 0 for a default-constructed object
            return _owned(np.zeros((0, self._c._dim), dtype=self._dtype()), self)
        self._check()
        if a.ndim == 0:
            return _owned(np.asarray(self._c(np.full(1, a))[:, 0]), self)
        if a.ndim != 1:
            raise ValueError("Invalid time array passed to a continuous_output object: the number of dimensions "
                             "must be 1, but it is {} instead".format(a.ndim))
        return _owned(np.ascontiguousarray(self._c(a.reshape(-1, 1))[:, :, 0]), self)

    def _dtype(self):
        tc = self._c._tcs
        return np.float64 if tc is None or tc.dtype == torch.float64 else np.float32

    @property
    def output(self):
        o = self._c.output
        return None if o is None else _owned(np.asarray(o[:, 0]), self)

    @property
    def times(self):
        t = self._c.times
        return None if t is None else _owned(np.asarray(t[:, 0]), self)

    @property
    def tcs(self):
        t = self._c.tcs
        return None if t is None else _owned(np.asarray(t[..., 0]), self)

    @property
    def bounds(self):
        self._check()
        t = self.times
        return (float(t[0]), float(t[-1]))

    @property
    def n_steps(self):
        self._check()
        return self._c.n_steps

    # Copies: the data are copied, attributes added from Python are shared by
    # a copy and deep-copied by a deep copy (heyoka/common_utils.hpp:96-150).
    def __copy__(self):
        new = continuous_output(_copy.copy(self._c))
        new.__dict__.update({k: v for k, v in self.__dict__.items() if k not in new.__dict__})
        return new

    def __deepcopy__(self, memo):
        new = continuous_output(_copy.deepcopy(self._c, memo))
        memo[id(self)] = new
        new.__dict__.update({k: _copy.deepcopy(v, memo) for k, v in self.__dict__.items() if k not in new.__dict__})
        return new

    def __repr__(self):
        if self._c._tcs is None:
            return "Default-constructed continuous_output"
        return "Direction : {}\nTime range: {}\nN of steps: {}\n".format(
            "forward" if self.bounds[1] >= self.bounds[0] else "backward", self.bounds, self.n_steps)


class _ScalarCallback:
    """A step callback of the scalar integrator, called by the one-lane batch
    with the scalar integrator as its argument (the object itself is called:
    no copies)."""

    def __init__(self, ta, cb):
        self._ta, self._cb = ta, cb

    def __call__(self, _batch):
        return self._cb(self._ta)

    def pre_hook(self, _batch):
        if hasattr(self._cb, "pre_hook"):
            self._cb.pre_hook(self._ta)


class taylor_adaptive:
    """Adaptive Taylor integrator of one trajectory (one GPU lane)."""

    def __init__(self, sys, state=[], time=0.0, pars=[], tol=0.0, high_accuracy=False,  # noqa: B006
                 compact_mode=False, t_events=[], nt_events=[], parallel_mode=False, *, fp_type=float,  # noqa: B006
                 **kwargs):
        from .events import batch_events_of_scalar, nt_event, t_event

        t_events, nt_events = list(t_events), list(nt_events)
        for e in t_events:
            if not isinstance(e, t_event):
                raise TypeError("the t_events argument must be a list of t_event objects")
        for e in nt_events:
            if not isinstance(e, nt_event):
                raise TypeError("the nt_events argument must be a list of nt_event objects")
        tb, nb = batch_events_of_scalar(t_events, nt_events, fp_type)
        np_dt, _ = _fp_of(fp_type)
        st = np.asarray(state)
        if st.ndim != 1:
            raise ValueError("The state vector passed to the constructor of a scalar integrator must be "
                             "one-dimensional, but it has {} dimensions".format(st.ndim))
        pa = np.asarray(pars)
        if pa.ndim != 1:
            raise ValueError("The parameter vector passed to the constructor of a scalar integrator must be "
                             "one-dimensional, but it has {} dimensions".format(pa.ndim))
        self._b = taylor_adaptive_batch(
            sys, st.reshape(-1, 1) if st.size else np.zeros((0, 1), dtype=np_dt),
            time=np.full(1, np_dt(time)), pars=pa.reshape(-1, 1) if pa.size else None, tol=tol,
            high_accuracy=high_accuracy, compact_mode=compact_mode, t_events=tb, nt_events=nb,
            parallel_mode=parallel_mode, fp_type=fp_type, **kwargs)
        self._b._scalar = self  # event callbacks are given the scalar integrator

    @classmethod
    def _wrap(cls, batch):
        new = object.__new__(cls)
        new._b = batch
        batch._scalar = new
        return new

    # ------------------------------------------------------------ state
    @property
    def state(self):
        return self._b.state[:, 0]

    @property
    def pars(self):
        return self._b.pars[:, 0]

    @property
    def time(self):
        return float(self._b.time[0])

    @time.setter
    def time(self, t):
        self._b.set_time(self._b._np_dt(t))

    @property
    def dtime(self):
        hi, lo = self._b.dtime
        return (float(hi[0]), float(lo[0]))

    @dtime.setter
    def dtime(self, p):
        hi, lo = p
        self._b.set_dtime(self._b._np_dt(hi), self._b._np_dt(lo))

    @property
    def tc(self):
        return self._b.tc[:, :, 0]

    @property
    def last_h(self):
        return float(self._b.last_h[0])

    @property
    def d_output(self):
        return self._b.d_output[:, 0]

    @property
    def tstate(self):
        return _owned(np.asarray(self._b.tstate[:, 0]), self)

    def __getattr__(self, name):
        # order, tol, dim, sys, decomposition, compact_mode, high_accuracy,
        # llvm_state, is_variational, vargs, vorder, n_orig_sv, fp_type, ...
        if name.startswith("_"):
            raise AttributeError(name)
        return getattr(self._b, name)

    @property
    def with_events(self):
        return self._b.with_events

    @property
    def t_events(self):
        from .events import _BoundEvent, t_event

        out = []
        for be in self._b._t_events:
            e = object.__new__(t_event)
            e.__dict__.update(be.__dict__)
            e._cb = None if be._cb is None else be._cb.cb
            out.append(_BoundEvent(self, e))
        return out

    @property
    def nt_events(self):
        from .events import _BoundEvent, nt_event

        out = []
        for be in self._b._nt_events:
            e = object.__new__(nt_event)
            e.__dict__.update(be.__dict__)
            e._cb = be._cb.cb
            out.append(_BoundEvent(self, e))
        return out

    @property
    def te_cooldowns(self):
        return self._b.te_cooldowns[0]

    def reset_cooldowns(self):
        self._b.reset_cooldowns()

    def get_vslice(self, order, component=None):
        return self._b.get_vslice(order, component)

    def get_mindex(self, i):
        return self._b.get_mindex(i)

    def eval_taylor_map(self, inputs):
        """The Taylor map at the displacements ``inputs`` (shape (n_vargs,));
        returns ``tstate`` (reference: heyoka/taylor_expose_integrator.cpp,
        checks as in heyoka/_test_var_integrator.py:68-110)."""
        b = self._b
        if b._vsys is None:
            raise ValueError("The integrator is not variational")
        m = len(b._vsys.vargs)
        overlap = ValueError("The array of inputs provided for the evaluation of a Taylor map may overlap with the "
                             "internal state of the integrator")
        if isinstance(inputs, torch.Tensor):
            if inputs.device.type == "cuda" and inputs.untyped_storage().data_ptr() == \
                    b._state.untyped_storage().data_ptr():
                raise overlap
            inputs = inputs.detach().cpu().numpy()
        if isinstance(inputs, np.ndarray) and np.shares_memory(inputs, b._tstate_buf()):
            raise overlap
        a = np.asarray(inputs)
        if isinstance(inputs, np.ndarray) and np.issubdtype(a.dtype, np.integer):
            raise TypeError("Invalid dtype detected for the inputs of a Taylor map evaluation: the expected dtype is "
                            "{}, but the dtype is {} instead".format(np.dtype(b._np_dt).name, a.dtype))
        if isinstance(inputs, np.ndarray) and not inputs.flags.c_contiguous:
            raise ValueError("Invalid inputs array detected in a Taylor map evaluation: the array is not C-style "
                             "contiguous, please consider using numpy.ascontiguousarray() to turn it into one")
        if a.ndim != 1:
            raise ValueError("The array of inputs provided for the evaluation of a Taylor map has {} dimensions, but "
                             "it must have 1 dimension instead".format(a.ndim))
        if a.size != m:
            raise ValueError("The array of inputs provided for the evaluation of a Taylor map has {} elements, but it "
                             "must have {} elements instead".format(a.size, m))
        b.eval_taylor_map(a.astype(b._np_dt).reshape(-1, 1))
        return self.tstate

    # ------------------------------------------------------------ stepping
    def step(self, max_delta_t=None, write_tc=False):
        if isinstance(max_delta_t, bool):
            write_tc, max_delta_t = max_delta_t, None
        self._b.step(None if max_delta_t is None else [max_delta_t], write_tc=write_tc)
        oc, h = self._b.step_res[0]
        return (oc, h)

    def step_backward(self, write_tc=False):
        self._b.step_backward(write_tc=write_tc)
        oc, h = self._b.step_res[0]
        return (oc, h)

    def update_d_output(self, t, rel_time=False):
        return self._b.update_d_output(self._b._np_dt(t), rel_time=rel_time)[:, 0]

    # ------------------------------------------------------------ propagation
    def _cbs(self, callback):
        if callback is None:
            return None
        return [_ScalarCallback(self, cb) for cb in _callbacks(callback)]

    def _res(self):
        oc, mn, mx, ns = self._b.propagate_res[0]
        return oc, mn, mx, ns

    def propagate_until(self, t, max_steps=0, max_delta_t=np.inf, callback=None, write_tc=False, c_output=False):
        self._b._check_prop_args(None, callback)
        c, _ = self._b.propagate_until(self._b._np_dt(t), max_steps=max_steps, max_delta_t=_mdt(max_delta_t),
                                       callback=self._cbs(callback), write_tc=write_tc, c_output=c_output)
        return self._res() + (None if c is None else continuous_output(c), callback)

    def propagate_for(self, delta_t, max_steps=0, max_delta_t=np.inf, callback=None, write_tc=False, c_output=False):
        self._b._check_prop_args(None, callback)
        c, _ = self._b.propagate_for(self._b._np_dt(delta_t), max_steps=max_steps, max_delta_t=_mdt(max_delta_t),
                                     callback=self._cbs(callback), write_tc=write_tc, c_output=c_output)
        return self._res() + (None if c is None else continuous_output(c), callback)

    def propagate_grid(self, grid, max_steps=0, max_delta_t=np.inf, callback=None):
        self._b._check_prop_args(None, callback)
        g = np.asarray(grid)
        if g.ndim != 1:
            raise ValueError("Invalid grid passed to the propagate_grid() method of a scalar integrator: the grid "
                             "must be one-dimensional, but it has {} dimensions".format(g.ndim))
        _, out = self._b.propagate_grid(g.reshape(-1, 1), max_steps=max_steps, max_delta_t=_mdt(max_delta_t),
                                        callback=self._cbs(callback))
        return self._res() + (callback, np.ascontiguousarray(out[:, :, 0]))

    # ------------------------------------------------------------ copies
    def __copy__(self):
        new = taylor_adaptive._wrap(_copy.copy(self._b))
        new.__dict__.update({k: v for k, v in self.__dict__.items() if k != "_b"})
        return new

    def __deepcopy__(self, memo):
        new = object.__new__(taylor_adaptive)
        memo[id(self)] = new
        new._b = _copy.deepcopy(self._b, memo)
        new._b._scalar = new
        for k, v in self.__dict__.items():
            if k != "_b":
                new.__dict__[k] = _copy.deepcopy(v, memo)
        return new

    def __getstate__(self):
        return dict(self.__dict__)

    def __setstate__(self, st):
        self.__dict__.update(st)
        self._b._scalar = self

    def __repr__(self):
        return repr(self._b).replace("Batch size              : 1\n", "")


def _mdt(max_delta_t):
    """The batch integrator's max_delta_t for a scalar one (+inf: none)."""
    v = float(max_delta_t)
    return [] if v == np.inf else v


# The reference's per-precision class names (the class here serves both).
continuous_output_dbl = continuous_output
continuous_output_flt = continuous_output

__all__ = ["continuous_output", "continuous_output_dbl", "continuous_output_flt", "taylor_adaptive", "taylor_outcome"]
