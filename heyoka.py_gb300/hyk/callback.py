"""Ready-made step callbacks (reference: heyoka/callback/__init__.py, the
C++ callbacks exposed by heyoka/expose_callbacks.cpp).

``angle_reducer(vars)``: after each step, the listed state variables are
reduced to the range [0, 2 pi) (reference changelog: "angle_reducer step
callback to automatically reduce angular state variables to the [0, 2 pi)
range").  On the GPU the reduction is one elementwise operation on the
device state between the propagation's steps.
"""

from __future__ import annotations

import copy as _copy
import math

import torch

from . import expr as _e

__all__ = ["angle_reducer"]

_TWO_PI = 2.0 * math.pi


class angle_reducer:
    def __init__(self, vars=()):  # noqa: A002 - the reference's argument name
        vs = [_e._ex(v) for v in vars]
        for v in vs:
            if v.kind != _e.VAR:
                raise ValueError("The angle_reducer callback accepts only variables, but '{}' is not".format(v))
        self._vars = vs
        self._idx = None

    def pre_hook(self, ta):
        names = [x.value for x, _ in ta.sys]
        idx = []
        for v in self._vars:
            if v.value not in names:
                raise ValueError(
                    "The variable '{}' is not a state variable of the integrator and cannot be reduced".format(v.value))
            idx.append(names.index(v.value))
        self._idx = idx

    def __call__(self, ta):
        if self._idx is None:
            self.pre_hook(ta)
        if self._idx:
            st = getattr(ta, "_b", ta)._state  # a scalar integrator's state is its one-lane batch's
            dt = st.dtype
            two_pi = torch.tensor(_TWO_PI, dtype=dt, device=st.device)
            rows = st[self._idx]
            red = torch.remainder(rows, two_pi)
            red = torch.where(red >= two_pi, red - two_pi, red)
            st[self._idx] = red
        return True

    def __repr__(self):
        return "Angle reducer: {}\n".format([str(v) for v in self._vars])

    def __copy__(self):
        new = angle_reducer(self._vars)
        new.__dict__.update({k: v for k, v in self.__dict__.items() if k not in ("_vars", "_idx")})
        return new

    def __deepcopy__(self, memo):
        new = angle_reducer(self._vars)
        for k, v in self.__dict__.items():
            if k not in ("_vars", "_idx"):
                new.__dict__[k] = _copy.deepcopy(v, memo)
        return new

    def __getstate__(self):
        return {k: v for k, v in self.__dict__.items() if k != "_idx"}

    def __setstate__(self, st):
        self.__dict__.update(st)
        self._idx = None
