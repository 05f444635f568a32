"""Ensemble propagations: ``ensemble_propagate_{until,for,grid}[_batch]``.

Same signatures, argument validation and return values as the reference
(heyoka/__init__.py:251-336, heyoka/_ensemble_impl.py:23-138): the generator
``gen(ta_copy, i)`` prepares iteration i from a copy of the template
integrator, and the result is a list with one ``(ta_i, ...)`` tuple per
iteration, exactly what the reference's thread or process pools return.

On the GPU the iterations are not separate tasks: the copies handed to the
generator are host-side (their tensors live on the CPU, so the generator only
sets state, parameters and time), then every iteration's lanes are
concatenated into one device batch, propagated by a single persistent kernel
launch and split back into per-iteration integrators.  The batch rules that
couple the lanes of one reference integrator (step limit for the whole batch,
last step of lanes that finished early) are applied per iteration.
``algorithm`` and ``max_workers`` are accepted for compatibility and do not
change the computation; ``chunksize`` is accepted with ``algorithm="process"``
only, as in the reference.

``devices=[d0, d1, ...]`` (no counterpart in the reference, whose workers are
host threads or processes: heyoka/_ensemble_impl.py:46-138) spreads the
iterations over several GPUs: contiguous ranges of iterations, one per entry,
each propagated as one device batch by a replica of the template on its GPU
(its own module there), the GPUs driven from one host thread each, and the
per-iteration results concatenated in iteration order.  Trajectories are
independent, so nothing is exchanged between GPUs.  A GPU named more than once
runs its ranges one after the other.
"""

from __future__ import annotations

import copy as _copy
from collections.abc import Iterable

import numpy as np
import torch

from .integrator import _callbacks, taylor_adaptive_batch


def _host_copy(ta):
    new = object.__new__(type(ta))
    for k, v in ta.__dict__.items():
        if isinstance(v, torch.Tensor):
            new.__dict__[k] = v.detach().to("cpu", copy=True)
        elif k == "_ev":
            new.__dict__[k] = None if v is None else {a: (b.detach().cpu() if isinstance(b, torch.Tensor) else b)
                                                      for a, b in v.items()}
        elif k in ("_prop", "_step_res", "_final_tc_mask", "_launch_events"):
            new.__dict__[k] = None
        else:
            new.__dict__[k] = v
    new.__dict__["_tdev"] = torch.device("cpu")
    return new


def _clone_host(tmpl):
    # A fresh host copy from the host template: CPU tensor clones only (the
    # device is read once per ensemble, not once per iteration).  Events are
    # deep-copied, as the reference's per-iteration deep copy does, so every
    # iteration has its own callback objects.
    new = object.__new__(type(tmpl))
    for k, v in tmpl.__dict__.items():
        if isinstance(v, torch.Tensor):
            new.__dict__[k] = v.clone()
        elif k in ("_t_events", "_nt_events"):
            new.__dict__[k] = _copy.deepcopy(v)
        elif k == "_ev":
            new.__dict__[k] = None if v is None else {a: (b.clone() if isinstance(b, torch.Tensor) else b)
                                                      for a, b in v.items()}
        else:
            new.__dict__[k] = v
    return new


def _split(t, n_iter, B):
    """Per-iteration contiguous blocks of a lane-minor device tensor (..., n_iter * B),
    made by one permuting copy instead of one copy per iteration."""
    lead = t.shape[:-1]
    v = t.reshape(*lead, n_iter, B)
    k = len(lead)
    return v.permute(k, *range(k), k + 1).contiguous()


def _validate(tp, arg, n_iter, kwargs):
    if not isinstance(n_iter, int):
        raise TypeError(
            "The n_iter parameter must be an integer, but an object of type {} was provided instead".format(
                type(n_iter)
            )
        )
    if n_iter < 0:
        raise ValueError("The n_iter parameter must be non-negative, but it is {} instead".format(n_iter))
    if tp in ("until", "for"):
        if isinstance(arg, Iterable):
            raise TypeError(
                "Cannot perform an ensemble propagate_until/for(): the final epoch/time interval must be a "
                "scalar, not an iterable object"
            )
    else:
        arg = np.array(arg)
        if arg.ndim != 1:
            raise ValueError(
                "Cannot perform an ensemble propagate_grid(): the input time grid must be one-dimensional, "
                "but instead it has {} dimensions".format(arg.ndim)
            )
    if "max_delta_t" in kwargs and isinstance(kwargs["max_delta_t"], Iterable):
        raise TypeError(
            'Cannot perform an ensemble propagate_until/for/grid(): the "max_delta_t" argument must be a '
            "scalar, not an iterable object"
        )
    algo = kwargs.pop("algorithm", "thread")
    if algo not in ("thread", "process"):
        raise ValueError(
            "The parallelisation algorithm must be one of {}, but '{}' was provided instead".format(
                ["thread", "process"], algo
            )
        )
    kwargs.pop("max_workers", None)
    if algo == "process":
        kwargs.pop("chunksize", None)
    return arg


def _ensemble_devices(tp, ta, arg, n_iter, gen, devices, kwargs):
    """The multi-GPU ensemble: iteration ranges per device (shard.partition),
    one host thread per distinct device, results in iteration order."""
    from concurrent.futures import ThreadPoolExecutor

    from . import shard
    from .integrator import _dev_index
    from .scalar import taylor_adaptive

    devs = [_dev_index(d) for d in devices]
    if not devs:
        raise ValueError("the devices argument must name at least one GPU")
    _validate(tp, arg, n_iter, dict(kwargs))  # the single-device path's errors, before any work
    if n_iter == 0:
        return []
    scalar = isinstance(ta, taylor_adaptive)
    base = ta._b if scalar else ta
    if not isinstance(base, taylor_adaptive_batch):
        raise TypeError("the GPU ensemble propagation needs a hyk.taylor_adaptive or hyk.taylor_adaptive_batch "
                        "template integrator")
    templates = {}
    for d in dict.fromkeys(devs):
        r = base if d == base._dev else base._replica(d)
        templates[d] = taylor_adaptive._wrap(r) if (scalar and r is not base) else (ta if r is base else r)
    ranges: dict = {}
    for (lo, hi), d in zip(shard.partition(n_iter, len(devs)), devs):
        if hi > lo:
            ranges.setdefault(d, []).append((lo, hi))

    def run(d):
        out = []
        for lo, hi in ranges[d]:
            part = _ensemble(tp, templates[d], arg, hi - lo, lambda c, i, lo=lo: gen(c, lo + i), **dict(kwargs))
            out.append((lo, part))
        return out

    with ThreadPoolExecutor(max_workers=len(ranges)) as ex:
        done = list(ex.map(run, list(ranges)))
    return [x for _, part in sorted((p for r in done for p in r), key=lambda p: p[0]) for x in part]


def _ensemble(tp, ta, arg, n_iter, gen, **kwargs):
    from .scalar import continuous_output, taylor_adaptive

    devices = kwargs.pop("devices", None)
    if devices is not None:
        return _ensemble_devices(tp, ta, arg, n_iter, gen, devices, kwargs)

    scalar = isinstance(ta, taylor_adaptive)  # a scalar template: one lane per iteration
    if scalar:
        ta = ta._b
    if not isinstance(ta, taylor_adaptive_batch):
        raise TypeError("the GPU ensemble propagation needs a hyk.taylor_adaptive or hyk.taylor_adaptive_batch "
                        "template integrator")
    arg = _validate(tp, arg, n_iter, kwargs)
    allowed = {"max_steps", "max_delta_t", "callback", "write_tc", "c_output"}
    if tp == "grid":
        allowed = {"max_steps", "max_delta_t", "callback"}
    for k in kwargs:
        if k not in allowed:
            raise TypeError("propagate_{}() got an unexpected keyword argument '{}'".format(tp, k))
    callback = kwargs.get("callback")
    if n_iter == 0:
        return []
    B = ta.batch_size
    tmpl = _host_copy(ta)
    scopies = None
    if scalar:
        scopies = [gen(taylor_adaptive._wrap(_clone_host(tmpl)), i) for i in range(n_iter)]
        for sc in scopies:
            if not isinstance(sc, taylor_adaptive):
                raise TypeError("the ensemble generator must return the integrator it was given")
        copies = [sc._b for sc in scopies]
    else:
        copies = [gen(_clone_host(tmpl), i) for i in range(n_iter)]
    for c in copies:
        if not isinstance(c, taylor_adaptive_batch) or c.batch_size != B or c._dec is not ta._dec:
            raise TypeError("the ensemble generator must return the integrator it was given")
    dev = ta._tdev
    # One device batch over all iterations.
    big = object.__new__(type(ta))
    big.__dict__.update(ta.__dict__)
    big._B = n_iter * B
    cat = lambda name: torch.cat([getattr(c, name).cpu() for c in copies], dim=-1).to(dev).contiguous()  # noqa: E731
    big._state = cat("_state")
    big._pars = cat("_pars")
    big._thi = cat("_thi")
    big._tlo = cat("_tlo")
    big._last_h = cat("_last_h")
    big._tc = cat("_tc")
    big._d_out = cat("_d_out")
    big._step_res = None
    big._prop = None
    big._final_tc_mask = None
    big._launch_events = None
    views = None
    if ta.with_events or callback is not None:
        # Per-iteration integrators whose tensors are views of the batch's,
        # for the event and step callbacks: a callback gets its iteration's
        # integrator (and, for events, its lane within it), and what it
        # writes (state, time) reaches the batch.
        views = []
        for i, c in enumerate(copies):
            sl = slice(i * B, (i + 1) * B)
            vi = object.__new__(type(ta))
            vi.__dict__.update(c.__dict__)
            vi._tdev = dev
            vi._state, vi._pars = big._state[:, sl], big._pars[:, sl]
            vi._thi, vi._tlo = big._thi[sl], big._tlo[sl]
            vi._ev = None
            views.append(vi)
    if ta.with_events:
        # Event buffers for the whole batch (the cooldown state of every
        # iteration's integrator carried over).
        big._ev = big._ev_alloc(16)
        big._ev["last"] = torch.cat([c._ev["last"] for c in copies], dim=-1).to(dev).contiguous()
        big._ev_route = (views, B)
    md = kwargs.get("max_delta_t", [])
    md = big._check_prop_args(md, callback)
    # Step callbacks: a deep copy per iteration, called with its iteration's
    # integrator (heyoka/_ensemble_impl.py:27-44).
    cb_copies = None if callback is None else [_copy.deepcopy(callback) for _ in range(n_iter)]
    if scalar and views is not None:
        for sc, vi in zip(scopies, views):
            sc._b = vi  # the callbacks see their iteration's scalar integrator
            vi._scalar = sc
    gcb = None if callback is None else [((scopies[i] if scalar else views[i]), _callbacks(cb_copies[i]))
                                         for i in range(n_iter)]
    ms = int(kwargs.get("max_steps", 0))
    if tp == "grid":
        g = torch.tensor(np.repeat(arg.astype(ta._np_dt), n_iter * B).reshape(-1, n_iter * B), device=dev)
        if not bool((g[0] == big._thi).all()):
            raise ValueError(
                "When invoking propagate_grid(), the first element of the time grid "
                "must match the current time coordinate"
            )
        res = big._run(g[-1].contiguous(), None, ms, md, grid=g, group=B, group_callbacks=gcb)
    else:
        tt = torch.full((n_iter * B,), float(ta._np_dt(arg)), dtype=ta._tdt, device=dev)
        if tp == "until":
            tf_hi, tf_lo = tt, None
        else:
            from .integrator import _dadd

            tf_hi, tf_lo = _dadd(big._thi, big._tlo, tt, torch.zeros_like(tt))
        res = big._run(tf_hi, tf_lo, ms, md, write_tc=bool(kwargs.get("write_tc", False)),
                       c_output=bool(kwargs.get("c_output", False)), group=B, group_callbacks=gcb)
    big._refresh_final_tc()
    parts = {name: _split(getattr(big, name), n_iter, B) for name in ("_state", "_pars", "_thi", "_tlo", "_last_h", "_tc", "_d_out")}
    prop = {k: (None if v is None else _split(v, n_iter, B)) for k, v in big._prop.items()}
    grid_np = None
    if tp == "grid":
        g = res["grid_out"].cpu().numpy()
        grid_np = g.reshape(g.shape[0], g.shape[1], n_iter, B)
    out = []
    for i, c in enumerate(copies):
        sl = slice(i * B, (i + 1) * B)
        ti = object.__new__(type(ta))
        # from the callbacks' view when there is one, so that what a callback
        # set on its integrator (attributes) is on the one returned
        ti.__dict__.update((views[i] if views is not None else c).__dict__)
        ti._tdev = dev
        for name, v in parts.items():
            ti.__dict__[name] = v[i]
        ti._prop = {k: (None if v is None else v[i]) for k, v in prop.items()}
        ti._step_res = None
        ti._final_tc_mask = None
        ti._launch_events = None
        if big._ev is not None:
            ti._ev = {a: (b[..., sl].contiguous() if isinstance(b, torch.Tensor) and a in ("last", "sign", "count")
                          else b) for a, b in big._ev.items()}
            for a in ("t_hi", "t_lo", "info"):
                ti._ev[a] = big._ev[a][:, sl].contiguous()
        ti.__dict__.pop("_ev_route", None)
        cb_i = None if cb_copies is None else cb_copies[i]
        if scalar:
            # the scalar integrator the generator returned, now on its result
            sc = scopies[i]
            sc._b = ti
            ti._scalar = sc
            r = ti.propagate_res[0]
            if tp == "grid":
                out.append((sc,) + tuple(r) + (cb_i, np.ascontiguousarray(grid_np[:, :, i, 0])))
            else:
                c_out = continuous_output(res["c_output"].lanes(sl)) if "c_output" in res else None
                out.append((sc,) + tuple(r) + (c_out, cb_i))
        elif tp == "grid":
            out.append((ti, cb_i, np.ascontiguousarray(grid_np[:, :, i, :])))
        else:
            c_out = None
            if "c_output" in res:
                c_out = res["c_output"].lanes(sl)
            out.append((ti, c_out, cb_i))
    return out


def ensemble_propagate_until(ta, t, n_iter, gen, **kwargs):
    return _ensemble("until", ta, t, n_iter, gen, **kwargs)


def ensemble_propagate_for(ta, delta_t, n_iter, gen, **kwargs):
    return _ensemble("for", ta, delta_t, n_iter, gen, **kwargs)


def ensemble_propagate_grid(ta, grid, n_iter, gen, **kwargs):
    return _ensemble("grid", ta, grid, n_iter, gen, **kwargs)


ensemble_propagate_until_batch = ensemble_propagate_until
ensemble_propagate_for_batch = ensemble_propagate_for
ensemble_propagate_grid_batch = ensemble_propagate_grid
