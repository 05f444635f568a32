"""``continuous_output_batch``: dense output over a whole batch propagation.

Mirrors the reference's continuous_output_batch (heyoka/taylor_expose_c_output.cpp:259-523):
``tcs`` of shape ``(n_steps, dim, order + 1, batch_size)`` (the Taylor
coefficients of every iteration, zero steps of lanes that finished early
included), ``times`` of shape ``(n_steps + 1, batch_size)`` (the start time,
then the end time of every iteration), and a call operator taking a time
batch ``(batch_size,)`` or a 2-D array of batches ``(n, batch_size)`` and
returning ``(dim, batch_size)`` / ``(n, dim, batch_size)``.

Evaluation runs on the GPU: for each lane the step containing t is found by a
batched binary search over the lane's end times (the last step whose start
time is <= t, clamped to the first/last step outside the range), and the
state polynomial is evaluated by Horner at the double-length offset from the
step start (libhyk's dense-output kernel).
"""

from __future__ import annotations

import copy as _copy

import numpy as np
import torch

from . import _lib
from .core import stream_handle
from .integrator import _owned


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _dsub_hi(ah, bh, bl):
    # hi part of (ah, 0) - (bh, bl) in double-length arithmetic
    s, e = _two_sum(ah, -bh)
    e = e + (0.0 - bl)
    return s + e


_DEFAULT_MSG = "Cannot use a default-constructed continuous_output_batch object"


class _DenseOutputState:
    """What ``llvm_state`` reports for a continuous output: the evaluator is
    libhyk's dense-output kernel, not JIT-compiled code."""

    ir = "hyk_dense_eval: Horner evaluation of the stored Taylor coefficients (CUDA, sm_103a)"

    def __repr__(self):
        return self.ir


class continuous_output_batch:
    def __init__(self, tcs=None, t_hi=None, t_lo=None, order=0, n_iter=None):
        if tcs is None:
            # a default-constructed object (reference: usable only after a propagation fills one)
            self._tcs = self._thi = self._tlo = None
            self._order, self._B, self._dim, self._out, self._nit = 0, 0, 0, None, None
            return
        self._tcs = tcs.contiguous()
        self._thi = t_hi.contiguous()
        self._tlo = t_lo.contiguous()
        self._order = int(order)
        self._dev = tcs.device
        self._B = t_hi.shape[1]
        self._dim = tcs.shape[1]
        self._out = None
        self._nit = n_iter
        n = self._tcs.shape[0]
        if n:
            # Search keys: start times of the steps, sign-normalised per lane
            # so that they are non-decreasing for backward propagations too.
            self._sgn = torch.where(self._thi[-1] < self._thi[0], -1.0, 1.0).to(tcs.dtype)
            self._keys = (self._thi[:n] * self._sgn).t().contiguous()  # (B, n)

    def _check(self):
        if self._tcs is None:
            raise ValueError(_DEFAULT_MSG)

    @property
    def llvm_state(self):
        return _DenseOutputState()

    @property
    def n_steps(self):
        self._check()
        return int(self._tcs.shape[0])

    @property
    def batch_size(self):
        return self._B

    @property
    def tcs(self):
        if self._tcs is None:
            return None
        return _owned(self._tcs.cpu().numpy(), self)

    @property
    def times(self):
        if self._thi is None:
            return None
        return _owned(self._thi.cpu().numpy(), self)

    @property
    def output(self):
        if self._out is None:
            return None
        return _owned(self._out.cpu().numpy(), self)

    @property
    def bounds(self):
        self._check()
        t = self._thi.cpu().numpy()
        return (np.array(t[0]), np.array(t[-1]))

    def _eval_row(self, t):
        n = self.n_steps
        idx = torch.searchsorted(self._keys, (t * self._sgn).view(self._B, 1).contiguous(), right=True).view(self._B)
        idx = (idx - 1).clamp(0, n - 1)
        lanes = torch.arange(self._B, device=self._dev)
        tc = self._tcs[idx, :, :, lanes].permute(1, 2, 0).contiguous()  # (dim, order+1, B)
        dt = _dsub_hi(t, self._thi[idx, lanes], self._tlo[idx, lanes]).contiguous()
        out = torch.empty((self._dim, self._B), dtype=self._tcs.dtype, device=self._dev)
        L = _lib.load()
        fn = L.hyk_dense_eval_f32 if self._tcs.dtype == torch.float32 else L.hyk_dense_eval
        with torch.cuda.device(self._dev):
            _lib.check(
                fn(
                    tc.data_ptr(), self._dim, self._order, self._B, self._B, dt.data_ptr(), out.data_ptr(),
                    stream_handle(self._dev.index),
                ),
                "hyk_dense_eval",
            )
        return out

    def __call__(self, tm=None, time=None):
        if tm is None:
            tm = time
        if self._tcs is None or self.n_steps == 0:
            raise ValueError(_DEFAULT_MSG)
        dt = self._tcs.dtype
        ndt = np.float32 if dt == torch.float32 else np.float64
        if isinstance(tm, torch.Tensor):
            t = tm.to(device=self._dev, dtype=dt)
        elif np.ndim(tm) == 0:
            # a scalar time applies to every lane (heyoka/taylor_expose_c_output.cpp:272-296)
            t = torch.full((self._B,), float(ndt(tm)), dtype=dt, device=self._dev)
        else:
            a = np.asarray(tm)
            if a.dtype != ndt:
                a = a.astype(ndt, casting="safe" if ndt == np.float64 else "same_kind")
            t = torch.tensor(a, dtype=dt, device=self._dev)
        if t.dim() not in (1, 2):
            raise ValueError(
                "Invalid time array passed to a continuous_output_batch object: the number of dimensions "
                "must be 1 or 2, but it is {} instead".format(t.dim())
            )
        if t.dim() == 1:
            if t.shape[0] != self._B:
                raise ValueError(
                    "Invalid time array passed to a continuous_output_batch object: the length must be {} "
                    "but it is {} instead".format(self._B, t.shape[0])
                )
            self._out = self._eval_row(t)
            return self.output
        if t.shape[1] != self._B:
            raise ValueError(
                "Invalid time array passed to a continuous_output_batch object: the number of columns must be "
                "{} but it is {} instead".format(self._B, t.shape[1])
            )
        rows = [self._eval_row(t[i].contiguous()) for i in range(t.shape[0])]
        if rows:
            self._out = rows[-1]
        res = torch.stack(rows) if rows else torch.empty((0, self._dim, self._B), dtype=dt)
        return _owned(res.cpu().numpy(), self)

    def lanes(self, sl):
        """The continuous output of a contiguous subset of lanes (one batch of
        an ensemble), trimmed to that subset's own number of iterations."""
        if self._nit is None:
            k = self.n_steps
        else:
            k = int(self._nit[sl].max().item()) if self._nit[sl].numel() else 0
        return continuous_output_batch(
            self._tcs[:k, :, :, sl].contiguous(), self._thi[: k + 1, sl].contiguous(),
            self._tlo[: k + 1, sl].contiguous(), self._order, None if self._nit is None else self._nit[sl],
        )

    def _clone(self):
        if self._tcs is None:
            return continuous_output_batch()
        new = continuous_output_batch(self._tcs.clone(), self._thi.clone(), self._tlo.clone(), self._order,
                                      None if self._nit is None else self._nit.clone())
        new._out = None if self._out is None else self._out.clone()
        return new

    def __copy__(self):
        # The data are copied (the reference's object is a value); attributes
        # added from Python are shared, as a shallow copy of the instance
        # dictionary (heyoka/taylor_expose_c_output.cpp:518-522, heyoka/common_utils.hpp:96-150).
        new = self._clone()
        new.__dict__.update({k: v for k, v in self.__dict__.items() if k not in new.__dict__})
        return new

    def __deepcopy__(self, memo):
        new = self._clone()
        memo[id(self)] = new
        new.__dict__.update({k: _copy.deepcopy(v, memo) for k, v in self.__dict__.items() if k not in new.__dict__})
        return new

    def __repr__(self):
        if self._tcs is None:
            return "Default-constructed continuous_output_batch"
        return "Directions : {}\nNumber of steps: {}\nBatch size: {}\n".format(
            "forward/backward per lane", self.n_steps, self._B
        )


# The reference's per-precision class names (the class here serves both).
continuous_output_batch_dbl = continuous_output_batch
continuous_output_batch_flt = continuous_output_batch
