"""Event detection for the batch integrator: ``nt_event_batch``,
``t_event_batch`` and ``event_direction``.

The classes mirror the reference's (heyoka/taylor_expose_events.cpp:202-311,
semantics in doc/notebooks/Batch mode overview.ipynb, tests in
heyoka/test.py:410-1000): the event equation, the callback (deep-copied at
construction), the direction and, for terminal events, the cooldown; same
reprs, errors, copy and pickle behaviour.

How they run here.  The event functions are decomposed together with the ODE
system, so every step's kernel has their Taylor coefficients, and the
kernel searches each one's polynomial over the step for roots (csrc/
hyk_events.h).  A terminal event ends the lane's step at its first root; the
roots of non-terminal events are recorded in device buffers.  The callbacks
run on the host after the kernel returns, in chronological order per lane:
a non-terminal callback ``cb(ta, t, d_sgn, bidx)`` once per recorded root,
a terminal callback ``cb(ta, d_sgn, bidx)`` for a lane stopped by its event,
whose ``True`` resumes the lane's propagation.  Unlike the reference, where a
non-terminal callback runs at the end of the step that found its root, here
it runs when the propagation (or the step) returns, with the integrator in
its state at that point.
"""

from __future__ import annotations

import copy as _copy
import enum

import numpy as np

from . import expr as _e
from . import s11n as _s11n

__all__ = ["event_direction", "nt_event", "nt_event_batch", "t_event", "t_event_batch"]


class event_direction(enum.IntEnum):
    """Direction of an event (reference: heyoka/core.cpp event_direction)."""

    negative = -1
    any = 0
    positive = 1


def _check_fp(fp_type):
    if fp_type not in (float, np.float64, np.float32):
        raise TypeError('The floating-point type "{}" is not recognized/supported'.format(fp_type))
    return "float" if fp_type is np.float32 else "double"


def _check_cb(cb):
    if not callable(cb):
        raise TypeError(
            "An object of type '{}' cannot be used as an event callback because it is not callable".format(
                str(type(cb))
            )
        )


def _dump_cb(cb):
    return _s11n.dumps(cb)


def _load_cb(blob):
    return _s11n.loads(blob)


class _EventBase:
    def __init__(self, ex, direction, fp_type):
        self._ctype = _check_fp(fp_type)
        self._ex = _e._ex(ex)
        self._dir = event_direction(direction)

    @property
    def expression(self):
        return self._ex

    @property
    def direction(self):
        return self._dir

    @property
    def callback(self):
        return self._cb

    def __getstate__(self):
        st = dict(self.__dict__)
        st["_cb"] = None if self._cb is None else _dump_cb(self._cb)
        return st

    def __setstate__(self, st):
        st = dict(st)
        cb = st.pop("_cb")
        self.__dict__.update(st)
        self._cb = None if cb is None else _load_cb(cb)

    def __copy__(self):
        new = object.__new__(type(self))
        new.__dict__.update(self.__dict__)
        return new

    def __deepcopy__(self, memo):
        new = object.__new__(type(self))
        memo[id(self)] = new
        for k, v in self.__dict__.items():
            new.__dict__[k] = _copy.deepcopy(v, memo)
        return new


class nt_event_batch(_EventBase):
    """Non-terminal event: ``callback(ta, t, d_sgn, bidx)`` at every root of
    ``ex`` (reference: heyoka/taylor_expose_events.cpp:202-250)."""

    def __init__(self, ex, callback, direction=event_direction.any, fp_type=float):
        super().__init__(ex, direction, fp_type)
        _check_cb(callback)
        self._cb = _copy.deepcopy(callback)

    def __repr__(self):
        return (
            "C++ datatype: {}\nEvent type: non-terminal\nEvent equation: {}\nEvent direction: "
            "event_direction::{}\n".format(self.__dict__.get("_ctype", "double"), self._ex, self._dir.name)
        )


class t_event_batch(_EventBase):
    """Terminal event: the step ends at the first root of ``ex``; optional
    ``callback(ta, d_sgn, bidx) -> bool`` (True resumes the propagation)
    (reference: heyoka/taylor_expose_events.cpp:252-311)."""

    def __init__(self, ex, callback=None, direction=event_direction.any, cooldown=-1.0, fp_type=float):
        super().__init__(ex, direction, fp_type)
        if callback is not None:
            _check_cb(callback)
        self._cb = None if callback is None else _copy.deepcopy(callback)
        self._cooldown = float(cooldown)

    @property
    def cooldown(self):
        return self._cooldown

    def __repr__(self):
        return (
            "C++ datatype: {}\nEvent type: terminal\nEvent equation: {}\nEvent direction: "
            "event_direction::{}\nWith callback: {}\nCooldown: {}\n".format(
                self.__dict__.get("_ctype", "double"), self._ex, self._dir.name, "yes" if self._cb is not None else "no",
                "auto" if self._cooldown < 0 else repr(self._cooldown),
            )
        )


class nt_event(_EventBase):
    """Non-terminal event of the scalar integrator: ``callback(ta, t, d_sgn)``
    at every root of ``ex`` (reference: heyoka/taylor_expose_events.cpp:202-250)."""

    def __init__(self, ex, callback, direction=event_direction.any, fp_type=float):
        super().__init__(ex, direction, fp_type)
        _check_cb(callback)
        self._cb = _copy.deepcopy(callback)

    __repr__ = nt_event_batch.__repr__


class t_event(_EventBase):
    """Terminal event of the scalar integrator: the step ends at the first
    root of ``ex``; optional ``callback(ta, d_sgn) -> bool`` (True resumes the
    propagation) (reference: heyoka/taylor_expose_events.cpp:252-311)."""

    def __init__(self, ex, callback=None, direction=event_direction.any, cooldown=-1.0, fp_type=float):
        super().__init__(ex, direction, fp_type)
        if callback is not None:
            _check_cb(callback)
        self._cb = None if callback is None else _copy.deepcopy(callback)
        self._cooldown = float(cooldown)

    cooldown = t_event_batch.cooldown
    __repr__ = t_event_batch.__repr__


class _ScalarNt:
    """A scalar event's non-terminal callback under the one-lane batch: the
    lane index is dropped."""

    def __init__(self, cb):
        self.cb = cb

    def __call__(self, ta, t, d_sgn, bidx):
        self.cb(ta, t, d_sgn)


class _ScalarT:
    """A scalar event's terminal callback under the one-lane batch."""

    def __init__(self, cb):
        self.cb = cb

    def __call__(self, ta, d_sgn, bidx):
        return self.cb(ta, d_sgn)


def batch_events_of_scalar(t_events, nt_events, fp_type):
    """The batch events that carry the scalar events (the callback objects
    are shared, not copied: the scalar events already hold their copies)."""
    tb, nb = [], []
    for e in t_events:
        be = object.__new__(t_event_batch)
        be.__dict__.update(e.__dict__)
        be._cb = None if e._cb is None else _ScalarT(e._cb)
        tb.append(be)
    for e in nt_events:
        be = object.__new__(nt_event_batch)
        be.__dict__.update(e.__dict__)
        be._cb = _ScalarNt(e._cb)
        nb.append(be)
    return tb, nb


class _BoundEvent:
    """An event as returned by the integrator's ``t_events``/``nt_events``:
    the integrator's own event object, which keeps the integrator alive."""

    __slots__ = ("_ta", "_ev")

    def __init__(self, ta, ev):
        self._ta = ta
        self._ev = ev

    def __getattr__(self, name):
        return getattr(self._ev, name)

    def __repr__(self):
        return repr(self._ev)


def callback_error(exc):
    return RuntimeError("An exception was raised by an event callback: {}".format(exc))


def check_bool_retval(ret):
    if isinstance(ret, (bool, np.bool_)):
        return bool(ret)
    raise RuntimeError(
        "An error occurred in the construction of the return value of an event callback: a bool was expected, "
        "but an object of type '{}' was returned instead".format(type(ret))
    )
