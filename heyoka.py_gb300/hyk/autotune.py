"""Kernel-configuration autotuner.

The code generator can run one system in several ways: one thread per
trajectory with the Taylor coefficients in shared memory (several block
sizes), one thread per trajectory with the coefficients in global memory, or
a team of 2..32 threads per trajectory.  Every configuration gives the same
bits; they differ in speed, and which is fastest depends on the system, the
order and the precision (the module constructor's occupancy estimate gets the
outer-solar-system problem wrong, for instance: it prefers a team of 16 over
the global-memory lane form, which is 1.2x faster).

``tune`` measures each configuration that compiles and fits on the device on
the same short workloads (the caller's initial states, replicated to fill the
GPU several times over, propagated for a fixed number of steps by the
persistent kernel, once without and once with a dense output grid of about
two points per step), keeps the fastest for each, and stores the choices
in a JSON cache
next to the compiled kernels (``$HYK_CACHE_DIR``, default ``~/.cache/hyk``)
keyed by the decomposition, the order, the precision, the compensated
summation flag and the device, so a later integrator of the same system
starts with it.  ``taylor_adaptive_batch(..., autotune=True)`` calls it.
"""

from __future__ import annotations

import json
import os
import threading
import time

import numpy as np
import torch

from . import _lib
from .core import _cache_lock, _modules, get_module
from .decompose import Decomposition, order_from_tol, taylor_decompose

_lock = threading.Lock()

# (team_size, global_jets, block_lanes) of the configurations tried; team
# size 0 and block size 0 let the module constructor choose.  The first entry
# is the constructor's own choice: another configuration replaces it only
# when it is faster by more than MARGIN (short measurements are noisy).
MARGIN = 1.03
DEFAULT_CANDIDATES = (
    (0, False, 0),
    (1, False, 0),
    (1, False, 64),
    (1, False, 128),
    (1, True, 0),
    (2, False, 0),
    (4, False, 0),
    (8, False, 0),
    (16, False, 0),
    (32, False, 0),
)


def cache_path():
    d = os.environ.get("HYK_CACHE_DIR") or os.path.join(os.environ.get("HOME", "/tmp"), ".cache", "hyk")
    return os.path.join(d, "autotune.json")


def cache_key(dec: Decomposition, order: int, device_name: str, float32: bool, high_accuracy: bool) -> str:
    return "{}|p{}|{}|{}|{}".format(dec.digest(), int(order), "f32" if float32 else "f64",
                                    "ha" if high_accuracy else "plain", device_name)


def _load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(key, entry):
    path = cache_path()
    with _lock:
        data = _load_cache()
        data[key] = entry
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".{}.tmp".format(os.getpid())
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def lookup(dec, order, device=0, float32=False, high_accuracy=False):
    """The cached choice for a system, or None."""
    key = cache_key(dec, order, torch.cuda.get_device_name(device), float32, high_accuracy)
    e = _load_cache().get(key)
    return None if e is None else dict(e["best"])


def _replicate(a, n):
    if a is None:
        return None
    a = np.asarray(a)
    reps = -(-n // a.shape[1])
    return np.ascontiguousarray(np.tile(a, (1, reps))[:, :n])


def tune(sys, state, pars=None, tol=0.0, *, fp_type=float, high_accuracy=False, device=None, steps=64,
         lanes=None, candidates=DEFAULT_CANDIDATES, use_cache=True, verbose=False):
    """Measure the kernel configurations of ``sys`` and return the fastest as
    ``result["best"] = {"team_size": T, "global_jets": bool, "block_lanes": b}``
    (propagate_until / propagate_for) and ``result["best_grid"]``
    (propagate_grid: the dense output reads every coefficient once per grid
    point, which favours coefficients in shared memory), together with the
    measurements (``result["trials"]``: one entry per configuration,
    trajectory-steps/s or the reason it was skipped).

    ``state`` (and ``pars``) are representative initial conditions, shape
    (n_eq, k) (and (n_pars, k)); they are replicated to ``lanes`` trajectories
    (default: four times the largest resident capacity of the
    configurations) and propagated for ``steps`` steps each."""
    from .integrator import _fp_of, taylor_adaptive_batch

    np_dt, t_dt = _fp_of(fp_type)
    f32 = t_dt == torch.float32
    dec = sys if isinstance(sys, Decomposition) else taylor_decompose(getattr(sys, "sys", sys))
    tol = float(np_dt(tol))
    if tol == 0.0:
        tol = float(np.finfo(np_dt).eps)
    order = order_from_tol(tol)
    dev = torch.cuda.current_device() if device is None else torch.device(device).index or 0
    key = cache_key(dec, order, torch.cuda.get_device_name(dev), f32, high_accuracy)
    if use_cache:
        e = _load_cache().get(key)
        if e is not None:
            out = dict(e)
            out["cached"] = True
            return out
    mods = []
    trials = []
    m_of = {}  # id(cfg) -> its module
    for T, gj, blk in candidates:
        cfg = {"team_size": int(T), "global_jets": bool(gj), "block_lanes": int(blk)}
        try:
            m = get_module(dec, order, dev, block_lanes=blk, team_size=T, high_accuracy=high_accuracy,
                           global_jets=gj, float32=f32)
        except _lib.HykError as exc:
            trials.append(dict(cfg, skipped=str(exc).splitlines()[0][:160]))
            continue
        i = m.info_dict()
        sig = (i["team_size"], i["smem_per_lane"] == 0, i["block_lanes"])
        if any(s == sig for s, _, _ in mods):
            trials.append(dict(cfg, skipped="same kernel as an earlier configuration"))
            continue
        cap = i["n_sm"] * i["ctas_per_sm"] * max(1, i["block_lanes"] // max(1, i["team_size"]))
        mods.append((sig, cfg, cap))
        m_of[id(cfg)] = m
    if not mods:
        raise _lib.HykError("autotune: no kernel configuration of this system fits the device")
    n = int(lanes) if lanes else min(max(c for _, _, c in mods) * 4, 1 << 20)
    st = _replicate(np.asarray(state, dtype=np_dt), n)
    pa = _replicate(None if pars is None else np.asarray(pars, dtype=np_dt), n)
    best = best_g = first = None
    grid = None
    for sig, cfg, cap in mods:
        ta = taylor_adaptive_batch(dec.sys, st, pars=pa, tol=tol, fp_type=fp_type, high_accuracy=high_accuracy,
                                   device=torch.device("cuda", dev), team_size=cfg["team_size"],
                                   global_jets=cfg["global_jets"], block_lanes=cfg["block_lanes"])
        s0 = ta._state.clone()
        if grid is None:
            # a grid of about two points per step of each lane (dense output
            # dominates grids of many points over short propagations)
            ta.step()
            h = ta._last_h.abs().double().clamp(min=1e-300)
            ta._state.copy_(s0)
            ta.set_time(0.0)
            frac = torch.linspace(0.0, 1.0, 2 * steps, dtype=torch.float64, device=h.device)
            grid = (frac.view(-1, 1) * (h * steps * 0.9).view(1, -1)).to(ta._tdt).contiguous()
        rate = rate_g = 0.0
        for rep in range(3):  # the first call warms up (module load, first launch)
            for g in (None, grid):
                ta._state.copy_(s0)
                ta.set_time(0.0)
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                if g is None:
                    ta.propagate_until(1e30, max_steps=steps)
                else:
                    ta.propagate_grid_tensor(g, max_steps=steps)
                torch.cuda.synchronize(dev)
                dt = time.perf_counter() - t0
                nst = int(ta.propagate_res_tensors["n_steps"].sum().item())
                if rep and g is None:
                    rate = max(rate, nst / dt)
                elif rep:
                    rate_g = max(rate_g, nst / dt)
        info = ta.module_info
        trials.append(dict(cfg, trajectory_steps_per_s=rate, grid_trajectory_steps_per_s=rate_g,
                           team=info["team_size"], jets="global" if info["smem_per_lane"] == 0 else "shared",
                           block=info["block_lanes"], ctas_per_sm=info["ctas_per_sm"]))
        if verbose:
            print("autotune", trials[-1], flush=True)
        if best is None or rate > best[0] * (MARGIN if best[1] is first else 1.0):
            best = (rate, cfg)
        if best_g is None or rate_g > best_g[0] * (MARGIN if best_g[1] is first else 1.0):
            best_g = (rate_g, cfg)
        if first is None:
            first = cfg
        del ta
    entry = {"best": best[1], "rate": best[0], "best_grid": best_g[1], "rate_grid": best_g[0], "trials": trials,
             "lanes": n, "steps": int(steps)}
    _forget_losers(dec, order, dev, [(m_of[id(best[1])]), m_of[id(best_g[1])]], [m for m in m_of.values()])
    if use_cache:
        _store_cache(key, entry)
    out = dict(entry)
    out["cached"] = False
    return out


def tune_call(ta, call, candidates=DEFAULT_CANDIDATES, repeats=2, apply=True, verbose=False):
    """Measure ``call(ta)`` (a propagation of the caller's own workload) with
    every kernel configuration of ``ta``'s system and keep the fastest.

    The state, time and parameters are restored before each run and at the
    end, so the call is timed on the same inputs each time (every
    configuration gives the same bits).  With ``apply`` the integrator then
    uses the fastest configuration for every call.  Returns ``{"best": cfg,
    "seconds": s, "trials": [...]}``; unlike ``tune`` nothing is cached (the
    measurement belongs to this workload)."""
    st0, th0, tl0, pa0 = ta._state.clone(), ta._thi.clone(), ta._tlo.clone(), ta._pars.clone()
    orig = (ta._mod, ta._mod_opts, ta.__dict__.get("_mod_grid"), ta.__dict__.get("_mod_grid_opts"))
    dev = ta._dev

    def restore():
        ta._state.copy_(st0)
        ta._thi.copy_(th0)
        ta._tlo.copy_(tl0)
        ta._pars.copy_(pa0)

    seen, trials, best, tried = [], [], None, []
    for T, gj, blk in candidates:
        cfg = {"team_size": int(T), "global_jets": bool(gj), "block_lanes": int(blk)}
        opts = dict(ta._mod_opts, team_size=int(T), global_jets=bool(gj), block_lanes=int(blk))
        try:
            m = get_module(ta._dec, ta._order, dev, **opts)
        except _lib.HykError as exc:
            trials.append(dict(cfg, skipped=str(exc).splitlines()[0][:160]))
            continue
        i = m.info_dict()
        sig = (i["team_size"], i["smem_per_lane"] == 0, i["block_lanes"])
        if sig in seen:
            trials.append(dict(cfg, skipped="same kernel as an earlier configuration"))
            continue
        seen.append(sig)
        tried.append(m)
        ta._mod, ta._mod_opts, ta._mod_grid, ta._mod_grid_opts = m, opts, None, None
        secs = float("inf")
        for rep in range(repeats + 1):  # the first run warms up
            restore()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            call(ta)
            torch.cuda.synchronize(dev)
            if rep:
                secs = min(secs, time.perf_counter() - t0)
        trials.append(dict(cfg, seconds=secs, team=i["team_size"],
                           jets="global" if i["smem_per_lane"] == 0 else "shared", block=i["block_lanes"]))
        if verbose:
            print("tune_call", trials[-1], flush=True)
        if best is None or secs < best[0]:
            best = (secs, cfg, m, opts)
    restore()
    if best is None:
        raise _lib.HykError("autotune: no kernel configuration of this system fits the device")
    keep = [best[2]] + ([] if apply else [orig[0]] + ([orig[2]] if orig[2] is not None else []))
    _forget_losers(ta._dec, ta._order, dev, keep, tried)
    if apply:
        ta._mod, ta._mod_opts, ta._mod_grid, ta._mod_grid_opts = best[2], best[3], None, None
    else:
        ta._mod, ta._mod_opts, ta._mod_grid, ta._mod_grid_opts = orig
    return {"best": best[1], "seconds": best[0], "trials": trials}


def _forget_losers(dec, order, dev, keep, tried):
    """Drop the measured modules that lost from the module cache (their device
    buffers, up to hundreds of MB for large systems in global memory, are
    freed once nothing uses them)."""
    keep_ids = {id(m) for m in keep}
    loser_ids = {id(m) for m in tried if id(m) not in keep_ids}
    with _cache_lock:
        for k in [k for k, m in _modules.items() if id(m) in loser_ids]:
            del _modules[k]
