"""Continuous-batching propagation server.

Requests (one ODE system, a block of trajectories, their parameters, start
and final times) arrive over time.  The server keeps every admitted
trajectory on the device and advances all of them together:

* one **lane pool** per ODE system: device arrays of a fixed lane capacity
  (state, parameters, double-length time and final time, and the propagation
  bookkeeping), sized from an HBM budget per pool;
* **admission by footprint**: a request is admitted as soon as its system's
  pool has free lanes for all its trajectories; otherwise it waits (FIFO);
* **time slices**: each pool runs the persistent propagation kernel over its
  active lanes for at most ``slice_iters`` steps per lane, then returns.
  Between slices the host admits new requests into free lanes, retires the
  requests whose lanes are all done (results copied back to the host, lanes
  freed) — lanes of many requests share one launch, and requests that arrive
  while others are on the GPU join the next slice;
* pools of different systems run on their own CUDA streams, so their slices
  overlap on the device.

Each lane's arithmetic does not depend on what else shares the launch or on
the slicing (the bookkeeping is stored exactly between slices), so a request's
result is bit-identical alone and in any mix.
"""

from __future__ import annotations

import ctypes
import time as _time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .core import get_module, lanes_struct
from .decompose import order_from_tol, taylor_decompose

_DONE = _lib.LANE_DONE | _lib.LANE_STOPPED


@dataclass
class Request:
    system: str
    state: np.ndarray  # (n_eq, n)
    t_final: float
    t0: float = 0.0
    pars: np.ndarray | None = None  # (n_pars, n)
    arrival: float = 0.0  # seconds from the start of the stream
    rid: int = -1


@dataclass
class Result:
    rid: int
    system: str
    state: np.ndarray
    time: np.ndarray
    outcome: np.ndarray
    n_steps: np.ndarray
    min_h: np.ndarray
    max_h: np.ndarray
    arrival: float
    admitted: float
    finished: float

    @property
    def latency(self):
        return self.finished - self.arrival


@dataclass
class _Active:
    req: Request
    slots: torch.Tensor  # device int64
    slots_host: np.ndarray
    admitted: float
    done: int = 0


class LanePool:
    """Device lanes of one ODE system."""

    def __init__(self, name, sys, tol, capacity, device, slice_iters):
        self.name = name
        self.dec = taylor_decompose(sys)
        self.order = order_from_tol(tol)
        self.dev = torch.device(device)
        self.mod = get_module(self.dec, self.order, self.dev.index)
        self.C = int(capacity)
        self.slice_iters = int(slice_iters)
        ne, npar, C = self.dec.n_eq, self.dec.n_pars, self.C
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.state = torch.zeros((ne, C), **f64)
        self.pars = torch.zeros((max(npar, 0), C), **f64)
        self.thi = torch.zeros(C, **f64)
        self.tlo = torch.zeros(C, **f64)
        self.tf = torch.zeros(C, **f64)
        self.a = {
            "rem_hi": torch.zeros(C, **f64),
            "rem_lo": torch.zeros(C, **f64),
            "outcome": torch.zeros(C, dtype=torch.int64, device=self.dev),
            "min_h": torch.zeros(C, **f64),
            "max_h": torch.zeros(C, **f64),
            "n_steps": torch.zeros(C, dtype=torch.int64, device=self.dev),
            "n_iter": torch.zeros(C, dtype=torch.int64, device=self.dev),
            "last_h": torch.zeros(C, **f64),
            "status": torch.full((C,), _DONE, dtype=torch.int32, device=self.dev),
        }
        self.owner = torch.full((C,), -1, dtype=torch.int64, device=self.dev)
        self.free = list(range(C - 1, -1, -1))  # stack of free lane indices
        self.active: dict = {}
        self.stream = torch.cuda.Stream(self.dev)
        self.ws = torch.zeros(64, dtype=torch.int32, device=self.dev)
        self.lane_steps = 0
        self.bytes_per_lane = (ne + npar + 16) * 8

    def n_active_lanes(self):
        return self.C - len(self.free)

    def admit(self, reqs, now):
        """Admit the longest prefix of `reqs` that fits in the free lanes (one
        host-to-device transfer and one scatter for all of them); returns
        how many were admitted."""
        k, need = 0, 0
        while k < len(reqs) and need + reqs[k].state.shape[1] <= len(self.free):
            need += reqs[k].state.shape[1]
            k += 1
        if k == 0:
            return 0
        batch = reqs[:k]
        slots_host = np.array([self.free.pop() for _ in range(need)], dtype=np.int64)
        ne, npar = self.dec.n_eq, self.dec.n_pars
        rows = ne + npar + 3  # state, pars, t0, tf, owner
        host = np.empty((rows, need))
        off = 0
        for r in batch:
            n = r.state.shape[1]
            host[:ne, off: off + n] = r.state
            if npar:
                host[ne: ne + npar, off: off + n] = np.asarray(r.pars, dtype=np.float64).reshape(npar, n)
            host[ne + npar, off: off + n] = r.t0
            host[ne + npar + 1, off: off + n] = r.t_final
            host[ne + npar + 2, off: off + n] = r.rid
            off += n
        with torch.cuda.stream(self.stream):
            pinned = torch.from_numpy(np.concatenate([host, slots_host.view(np.float64).reshape(1, -1)])).pin_memory()
            dev = pinned.to(self.dev, non_blocking=True)
            slots = dev[-1].view(torch.int64)
            self.state[:, slots] = dev[:ne]
            if npar:
                self.pars[:, slots] = dev[ne: ne + npar]
            t0, tf = dev[ne + npar], dev[ne + npar + 1]
            self.thi[slots] = t0
            self.tlo[slots] = 0.0
            self.tf[slots] = tf
            # remaining time = tf - t0 in double-length arithmetic (as the
            # propagation initialisation kernel computes it)
            s = tf - t0
            bb = s - tf
            e = (tf - (s - bb)) + (-t0 - bb)
            e = e + 0.0
            hi = s + e
            lo = e - (hi - s)
            self.a["rem_hi"][slots] = hi
            self.a["rem_lo"][slots] = lo
            self.a["min_h"][slots] = float("inf")
            self.a["max_h"][slots] = 0.0
            self.a["n_steps"][slots] = 0
            self.a["n_iter"][slots] = 0
            self.a["last_h"][slots] = 0.0
            self.a["outcome"][slots] = int(-4294967299)
            zero = (hi == 0) & (lo == 0)
            self.a["status"][slots] = torch.where(zero, _lib.LANE_DONE, 0).to(torch.int32)
            self.owner[slots] = dev[ne + npar + 2].to(torch.int64)
        off = 0
        for r in batch:
            n = r.state.shape[1]
            self._ensure_counter(r.rid)
            self.active[r.rid] = _Active(r, slots[off: off + n], slots_host[off: off + n], now)
            off += n
        return k

    def _ensure_counter(self, rid):
        if getattr(self, "cnt", None) is None or rid + 1 >= self.cnt.numel():
            n = max(1024, 2 * (rid + 2))
            self.cnt = torch.zeros(n, dtype=torch.int32, device=self.dev)
            self.cnt_host = torch.zeros(n, dtype=torch.int32).pin_memory()

    def launch_slice(self):
        """Advance every active lane by up to slice_iters steps (async on the pool's stream)."""
        if not self.active:
            return
        L = _lib.load()
        with torch.cuda.stream(self.stream):
            # the lanes of the active requests (finished ones are skipped by the kernel)
            order = torch.cat([act.slots for act in self.active.values()]).contiguous()
            self._order = order
            a = self.a
            d = _lib.hyk_prop_t(
                self.tf.data_ptr(), None, None, 0, None, 0, None, None, None, None, 0,
                a["rem_hi"].data_ptr(), a["rem_lo"].data_ptr(), a["outcome"].data_ptr(), a["min_h"].data_ptr(),
                a["max_h"].data_ptr(), a["n_steps"].data_ptr(), a["n_iter"].data_ptr(), None,
                a["last_h"].data_ptr(), None, a["status"].data_ptr(), order.data_ptr(), order.numel(),
                None, None, None, 0, self.slice_iters,
            )
            lanes = lanes_struct(self.state, self.pars, self.thi, self.tlo)
            with torch.cuda.device(self.dev):
                _lib.check(
                    L.hyk_propagate(self.mod.handle, lanes, d, _lib.HYK_MODE_PERSISTENT, self.ws.data_ptr(), 256, 0,
                                    None, ctypes.c_void_p(self.stream.cuda_stream)),
                    "hyk_propagate",
                )
            # per-request count of finished lanes (no host synchronisation:
            # a scatter-add into a counter per request id, copied back async)
            fin = ((self.owner >= 0) & ((self.a["status"] & _DONE) != 0)).to(torch.int32)
            self.cnt.zero_()
            self.cnt.scatter_add_(0, self.owner + 1, fin)
            self.cnt_host.copy_(self.cnt, non_blocking=True)
            self._evt = torch.cuda.Event()
            self._evt.record(self.stream)

    def retire(self, now_fn):
        """Collect the requests whose lanes are all done and free their lanes.

        All finished requests of this slice are gathered by one device gather
        and copied back in one transfer."""
        if not self.active or getattr(self, "_evt", None) is None:
            return []
        self._evt.synchronize()
        self._evt = None
        counts = self.cnt_host.numpy()
        done = [rid for rid, act in self.active.items() if counts[rid + 1] >= act.req.state.shape[1]]
        if not done:
            return []
        acts = [self.active[rid] for rid in done]
        with torch.cuda.stream(self.stream):
            slots = torch.cat([a.slots for a in acts])
            ne = self.dec.n_eq
            packed = torch.cat([
                self.state[:, slots],
                self.thi[slots].view(1, -1),
                self.a["outcome"][slots].view(1, -1).view(torch.float64),
                self.a["n_steps"][slots].view(1, -1).view(torch.float64),
                self.a["min_h"][slots].view(1, -1),
                self.a["max_h"][slots].view(1, -1),
            ])
            host = torch.empty(packed.shape, dtype=torch.float64).pin_memory()
            host.copy_(packed, non_blocking=True)
            self.owner[slots] = -1
            self.a["status"][slots] = _DONE
            ev = torch.cuda.Event()
            ev.record(self.stream)
        ev.synchronize()
        h = host.numpy()
        t = now_fn()
        out, off = [], 0
        for rid, act in zip(done, acts):
            n = act.req.state.shape[1]
            blk = h[:, off: off + n]
            off += n
            ns = blk[ne + 2].copy().view(np.int64)
            out.append(Result(rid, self.name, blk[:ne].copy(), blk[ne].copy(), blk[ne + 1].copy().view(np.int64), ns,
                              blk[ne + 3].copy(), blk[ne + 4].copy(), arrival=act.req.arrival, admitted=act.admitted,
                              finished=t))
            self.lane_steps += int(ns.sum())
            self.free.extend(act.slots_host.tolist())
            del self.active[rid]
        return out


class Server:
    """Continuous-batching server over a set of ODE systems.

    ``systems``: name -> (sys, tol).  ``hbm_budget``: bytes of lane state per
    system pool (admission by footprint).  ``slice_iters``: steps per lane per
    kernel launch between admission rounds."""

    def __init__(self, systems, hbm_budget=2 << 30, slice_iters=64, device="cuda:0", max_lanes=1 << 21):
        self.pools = {}
        for name, (sys, tol) in systems.items():
            dec = taylor_decompose(sys)
            bpl = (dec.n_eq + dec.n_pars + 16) * 8
            cap = int(min(max_lanes, hbm_budget // bpl))
            self.pools[name] = LanePool(name, sys, tol, cap, device, slice_iters)

    def run(self, requests, realtime=True):
        """Serve `requests` (with arrival times in seconds); returns the results
        in completion order.  With ``realtime`` the arrivals follow the wall
        clock; otherwise each request is available from the start."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(reqs):
            if r.rid < 0:
                r.rid = i
        waiting = {name: [] for name in self.pools}
        results = []
        t_start = _time.perf_counter()

        def now():
            return _time.perf_counter() - t_start

        i = 0
        n = len(reqs)
        while i < n or any(waiting[k] for k in waiting) or any(p.active for p in self.pools.values()):
            t = now()
            while i < n and (not realtime or reqs[i].arrival <= t):
                waiting[reqs[i].system].append(reqs[i])
                i += 1
            for name, pool in self.pools.items():
                q = waiting[name]
                if q:
                    k = pool.admit(q, now())
                    if k:
                        del q[:k]
            busy = False
            for pool in self.pools.values():
                if pool.active:
                    pool.launch_slice()
                    busy = True
            for pool in self.pools.values():
                results.extend(pool.retire(now))
            if not busy and i < n:
                dt = reqs[i].arrival - now()
                if dt > 0:
                    _time.sleep(min(dt, 0.01))
        return results

    def trajectory_steps(self):
        return sum(p.lane_steps for p in self.pools.values())


def latency_stats(results):
    lat = np.array([r.latency for r in results])
    if lat.size == 0:
        return {}
    return {
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "mean_ms": float(lat.mean() * 1e3),
        "n": int(lat.size),
    }
