"""Continuous-batching propagation server.

Requests (one ODE system, a block of trajectories, their parameters, start
and final times) arrive over time.  The server keeps every admitted
trajectory on the device and advances all of them together:

* one **lane pool** per ODE system: device arrays of a fixed lane capacity
  (state, parameters, double-length time and final time, and the propagation
  bookkeeping), sized from an HBM budget per pool;
* **admission by footprint**: a request is admitted as soon as its system's
  pool has free lanes for all its trajectories; otherwise it waits (FIFO);
* **time slices**: each pool runs the persistent propagation kernel over the
  lanes of its active requests for a bounded number of steps per lane.  The
  number is chosen per slice so that the slice lasts about one time quantum
  (``quantum_ms``) from the pool's measured step rate and its number of
  active lanes per resident thread: few active lanes get many steps per
  slice (a long request then runs nearly as fast as alone), many active
  lanes get few (a new request never waits long for the next slice);
* **pipelining**: when a pool holds more lanes than it has resident threads,
  two slices are queued on its stream, so the device works on the next slice
  while the host admits and retires; a lightly loaded pool keeps one, so a
  new request waits for one slice at most.  The host never blocks on a slice;
* **retirement**: after each slice the per-request count of finished lanes
  (one scatter-add over the slice's lanes) comes back asynchronously; the
  requests whose lanes are all done are gathered by one device gather and
  copied back in one transfer, and their lanes are freed;
* pools of different systems run on their own CUDA streams, so their slices
  overlap on the device.

Each lane's arithmetic does not depend on what else shares the launch or on
the slicing (the bookkeeping is stored exactly between slices), so a request's
result is bit-identical alone and in any mix.
"""

from __future__ import annotations

import ctypes
import time as _time
from collections import deque
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
    slots_host: np.ndarray
    admitted: float
    retiring: bool = False


@dataclass
class _Slice:
    t0: torch.cuda.Event
    t1: torch.cuda.Event
    done: torch.cuda.Event  # after the finished-lane counts were copied
    counts: torch.Tensor  # pinned host copy of the per-request finished-lane counters
    iters: int
    waves: int


@dataclass
class _Gather:
    event: torch.cuda.Event
    host: torch.Tensor
    acts: list


class LanePool:
    """Device lanes of one ODE system.

    The per-lane arrays live in two tables so that admitting and retiring a
    batch of requests is a handful of device operations: a float64 table
    (state rows, parameter rows, then time hi/lo, final time, remaining time
    hi/lo, min |h|, max |h|, last h) and an int64 table (outcome, step count,
    iteration count, owning request), plus the int32 lane status."""

    def __init__(self, name, sys, tol, capacity, device, slice_iters, quantum_s=0.002, max_requests=1 << 16):
        self.name = name
        self.dec = taylor_decompose(sys)
        self.order = order_from_tol(tol)
        self.dev = torch.device(device)
        self.mod = get_module(self.dec, self.order, self.dev.index)
        info = self.mod.info_dict()
        self.resident = max(1, info["n_sm"] * info["ctas_per_sm"] * (info["block_lanes"] // info["team_size"]))
        self.C = int(capacity)
        self.max_iters = max(1, int(slice_iters))
        self.quantum = float(quantum_s)
        # Seconds per step of one resident lane.  Floor: a warp alone on an SM
        # sub-partition is bound by that sub-partition's FP64 unit, about
        # 20 ns per algorithmic flop of the step (a Kepler step, 2668 flop,
        # takes ~55 us alone); above it, the estimate follows the measured
        # slices, rising at once and decaying slowly (a slice whose lanes
        # finish early would otherwise lower it and make the next slice of
        # long lanes overrun the quantum).
        self.tau_floor = 2e-8 * float(info["flops_per_step"])
        self.tau = self.tau_floor
        ne, npar, C = self.dec.n_eq, self.dec.n_pars, self.C
        b = ne + npar
        self.R = {"thi": b, "tlo": b + 1, "tf": b + 2, "rem_hi": b + 3, "rem_lo": b + 4, "min_h": b + 5,
                  "max_h": b + 6, "last_h": b + 7}
        self.RF = b + 8
        self.F = torch.zeros((self.RF, C), dtype=torch.float64, device=self.dev)
        self.I = torch.zeros((4, C), dtype=torch.int64, device=self.dev)  # outcome, n_steps, n_iter, owner
        self.I[3].fill_(-1)
        self.status = torch.full((C,), _DONE, dtype=torch.int32, device=self.dev)
        self.state, self.pars = self.F[:ne], self.F[ne:b]
        self.thi, self.tlo, self.tf = self.F[b], self.F[b + 1], self.F[b + 2]
        self.a = {k: self.F[r] for k, r in self.R.items() if k not in ("thi", "tlo", "tf")}
        self.a.update(outcome=self.I[0], n_steps=self.I[1], n_iter=self.I[2], status=self.status)
        self.owner = self.I[3]
        self.free_arr = np.arange(C - 1, -1, -1, dtype=np.int64)  # stack of free lane indices
        self.n_free = C
        self.active: dict = {}
        self.stream = torch.cuda.Stream(self.dev)
        # results are gathered on a stream of their own, so that they do not
        # wait for the slice queued behind the one that finished them
        self.io = torch.cuda.Stream(self.dev)
        self.ws = torch.zeros(64, dtype=torch.int32, device=self.dev)
        self.lane_steps = 0
        self.bytes_per_lane = (self.RF + 4) * 8 + 4
        self.cnt = torch.zeros(int(max_requests) + 1, dtype=torch.int32, device=self.dev)
        self.inflight: deque = deque()
        self.gathers: deque = deque()
        self._order = None  # device list of the active lanes (rebuilt when the active set changes)
        self._order_host = None
        self._dirty = True

    @property
    def free(self):
        return self.free_arr[: self.n_free]

    def n_active_lanes(self):
        return self.C - self.n_free

    def reserve_requests(self, n):
        if n + 1 > self.cnt.numel():
            with torch.cuda.stream(self.stream):
                self.cnt = torch.zeros(n + 1, dtype=torch.int32, device=self.dev)

    def admit(self, reqs, now):
        """Admit the longest prefix of `reqs` that fits in the free lanes: the
        lanes' initial rows are assembled on the host, copied in one transfer
        and scattered by three indexed writes; returns how many requests were
        admitted."""
        k, need = 0, 0
        while k < len(reqs) and need + reqs[k].state.shape[1] <= self.n_free:
            need += reqs[k].state.shape[1]
            k += 1
        if k == 0:
            return 0
        batch = reqs[:k]
        self.reserve_requests(max(r.rid for r in batch) + 1)
        slots_host = self.free_arr[self.n_free - need: self.n_free].copy()
        self.n_free -= need
        ne, npar, RF, R = self.dec.n_eq, self.dec.n_pars, self.RF, self.R
        blk = np.empty((RF + 6, need))
        ints = blk[RF:].view(np.int64)  # outcome, n_steps, n_iter, owner, status, slot
        off = 0
        for r in batch:
            n = r.state.shape[1]
            blk[:ne, off: off + n] = r.state
            if npar:
                blk[ne: ne + npar, off: off + n] = np.asarray(r.pars, dtype=np.float64).reshape(npar, n)
            blk[R["thi"], off: off + n] = r.t0
            blk[R["tf"], off: off + n] = r.t_final
            ints[3, off: off + n] = r.rid
            off += n
        t0, tf = blk[R["thi"]], blk[R["tf"]]
        # remaining time = tf - t0 in double-length arithmetic (the operations
        # of the propagation initialisation kernel, in IEEE double)
        s = tf - t0
        bb = s - tf
        e = (tf - (s - bb)) + (-t0 - bb)
        e = e + 0.0
        hi = s + e
        lo = e - (hi - s)
        blk[R["tlo"]] = 0.0
        blk[R["rem_hi"]], blk[R["rem_lo"]] = hi, lo
        blk[R["min_h"]], blk[R["max_h"]], blk[R["last_h"]] = np.inf, 0.0, 0.0
        ints[0] = -4294967299
        ints[1] = 0
        ints[2] = 0
        ints[4] = np.where((hi == 0) & (lo == 0), _lib.LANE_DONE, 0)
        ints[5] = slots_host
        with torch.cuda.stream(self.stream):
            dev = torch.from_numpy(blk).pin_memory().to(self.dev, non_blocking=True)
            di = dev[RF:].view(torch.int64)
            slots = di[5]
            self.F[:, slots] = dev[:RF]
            self.I[:, slots] = di[:4]
            self.status[slots] = di[4].to(torch.int32)
        off = 0
        for r in batch:
            n = r.state.shape[1]
            self.active[r.rid] = _Active(r, slots_host[off: off + n], now)
            off += n
        self._dirty = True
        return k

    def _lanes_of_active(self):
        if self._dirty:
            acts = [a.slots_host for a in self.active.values() if not a.retiring]
            self._order_host = np.concatenate(acts) if acts else np.zeros(0, dtype=np.int64)
            with torch.cuda.stream(self.stream):
                self._order = torch.from_numpy(self._order_host).pin_memory().to(self.dev, non_blocking=True)
            self._dirty = False
        return self._order

    def launch_slice(self):
        """Queue one slice over the lanes of the active requests (async on the
        pool's stream); the steps per lane aim at one time quantum."""
        order = self._lanes_of_active()
        n = int(order.numel())
        if n == 0:
            return False
        waves = -(-n // self.resident)
        # at least a few steps per lane, so that a heavily loaded pool's
        # slices are not dominated by their fixed costs
        iters = int(min(self.max_iters, max(4, self.quantum / (self.tau * waves))))
        L = _lib.load()
        with torch.cuda.stream(self.stream):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a = self.a
            d = _lib.hyk_prop_t(
                self.tf.data_ptr(), None, None, 0, None, 0, None, None, None, None, 0,
                a["rem_hi"].data_ptr(), a["rem_lo"].data_ptr(), a["outcome"].data_ptr(), a["min_h"].data_ptr(),
                a["max_h"].data_ptr(), a["n_steps"].data_ptr(), a["n_iter"].data_ptr(), None,
                a["last_h"].data_ptr(), None, a["status"].data_ptr(), order.data_ptr(), n,
                None, None, None, 0, iters,
            )
            lanes = lanes_struct(self.state, self.pars, self.thi, self.tlo)
            t0.record(self.stream)
            with torch.cuda.device(self.dev):
                _lib.check(
                    L.hyk_propagate(self.mod.handle, lanes, d, _lib.HYK_MODE_PERSISTENT, self.ws.data_ptr(), 256, 0,
                                    None, ctypes.c_void_p(self.stream.cuda_stream)),
                    "hyk_propagate",
                )
            t1.record(self.stream)
            # per-request count of finished lanes over this slice's lanes
            own = self.owner.index_select(0, order)
            fin = ((self.status.index_select(0, order) & _DONE) != 0).to(torch.int32)
            self.cnt.zero_()
            self.cnt.scatter_add_(0, own + 1, fin)
            counts = torch.empty(self.cnt.shape, dtype=torch.int32).pin_memory()
            counts.copy_(self.cnt, non_blocking=True)
            done_ev = torch.cuda.Event()
            done_ev.record(self.stream)
        self.inflight.append(_Slice(t0, t1, done_ev, counts, iters, waves))
        self.last_waves = waves
        return True

    def depth(self):
        """Slices to keep queued: two when the pool holds more lanes than its
        resident threads (the device then never waits for the host), one
        otherwise (a new request then waits for one slice at most)."""
        return 2 if getattr(self, "last_waves", 1) > 1 else 1

    def poll(self, now_fn, block=False):
        """Process the slices and result gathers that have completed (all of
        them in order, waiting for them with ``block``); returns the finished
        requests' results."""
        out = []
        while self.inflight and (block or self.inflight[0].done.query()):
            sl = self.inflight.popleft()
            sl.done.synchronize()
            ms = sl.t0.elapsed_time(sl.t1)
            if ms > 0:
                tau = ms * 1e-3 / (sl.iters * sl.waves)
                self.tau = max(self.tau_floor, tau if tau > self.tau else 0.9 * self.tau + 0.1 * tau)
            counts = sl.counts.numpy()
            done = [rid for rid, act in self.active.items()
                    if not act.retiring and counts[rid + 1] >= act.req.state.shape[1]]
            if done:
                self._gather(done, sl.done)
        while self.gathers and (block or self.gathers[0].event.query()):
            g = self.gathers.popleft()
            g.event.synchronize()
            out.extend(self._results(g, now_fn()))
        return out

    def _gather(self, done, after):
        """Copy the finished requests' lanes back (on the io stream, after the
        slice event `after` that counted them; a running later slice leaves
        finished lanes untouched) and queue the release of their lanes on the
        pool stream."""
        acts = [self.active[rid] for rid in done]
        for a in acts:
            a.retiring = True
        self._dirty = True
        slots_h = torch.from_numpy(np.concatenate([a.slots_host for a in acts])).pin_memory()
        with torch.cuda.stream(self.io):
            self.io.wait_event(after)
            slots = slots_h.to(self.dev, non_blocking=True)
            packed = torch.cat([self.F[:, slots], self.I[:3, slots].view(torch.float64)])
            host = torch.empty(packed.shape, dtype=torch.float64).pin_memory()
            host.copy_(packed, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.io)
        with torch.cuda.stream(self.stream):
            self.stream.wait_event(ev)  # the reads above come before any reuse of the lanes
            slots2 = slots_h.to(self.dev, non_blocking=True)
            self.owner[slots2] = -1
            self.status[slots2] = _DONE
        self.gathers.append(_Gather(ev, host, acts))

    def _results(self, g, t):
        h = g.host.numpy()
        ne, RF, R = self.dec.n_eq, self.RF, self.R
        ints = h[RF:].view(np.int64)
        out, off = [], 0
        for act in g.acts:
            n = act.req.state.shape[1]
            sl = slice(off, off + n)
            off += n
            ns = ints[1, sl].copy()
            out.append(Result(act.req.rid, self.name, h[:ne, sl].copy(), h[R["thi"], sl].copy(), ints[0, sl].copy(),
                              ns, h[R["min_h"], sl].copy(), h[R["max_h"], sl].copy(), arrival=act.req.arrival,
                              admitted=act.admitted, finished=t))
            self.lane_steps += int(ns.sum())
            # the lanes are reused only by admissions queued after this gather
            k = act.slots_host.size
            self.free_arr[self.n_free: self.n_free + k] = act.slots_host
            self.n_free += k
            del self.active[act.req.rid]
        return out

    def busy(self):
        return bool(self.active or self.inflight or self.gathers)


class Server:
    """Continuous-batching server over a set of ODE systems.

    ``systems``: name -> (sys, tol).  ``hbm_budget``: bytes of lane state per
    system pool (admission by footprint).  ``slice_iters``: the most steps
    per lane in one slice; ``quantum_ms``: the target duration of a slice."""

    def __init__(self, systems, hbm_budget=2 << 30, slice_iters=1024, device="cuda:0", max_lanes=1 << 21,
                 quantum_ms=2.0):
        self.pools = {}
        for name, (sys, tol) in systems.items():
            dec = taylor_decompose(sys)
            bpl = (dec.n_eq + dec.n_pars + 16) * 8
            cap = int(min(max_lanes, hbm_budget // bpl))  # lanes that fit the pool's HBM budget
            self.pools[name] = LanePool(name, sys, tol, cap, device, slice_iters, quantum_ms * 1e-3)

    def run(self, requests, realtime=True):
        """Serve `requests` (with arrival times in seconds); returns the results
        in completion order.  With ``realtime`` the arrivals follow the wall
        clock; otherwise each request is available from the start."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(reqs):
            if r.rid < 0:
                r.rid = i
        top = max((r.rid for r in reqs), default=0) + 1
        for p in self.pools.values():
            p.reserve_requests(top)
        waiting = {name: [] for name in self.pools}
        results = []
        t_start = _time.perf_counter()

        def now():
            return _time.perf_counter() - t_start

        i = 0
        n = len(reqs)
        while i < n or any(waiting.values()) or any(p.busy() for p in self.pools.values()):
            t = now()
            while i < n and (not realtime or reqs[i].arrival <= t):
                waiting[reqs[i].system].append(reqs[i])
                i += 1
            progressed = False
            for name, pool in self.pools.items():
                q = waiting[name]
                if q:
                    k = pool.admit(q, now())
                    if k:
                        del q[:k]
                        progressed = True
                while len(pool.inflight) < pool.depth() and pool.launch_slice():
                    progressed = True
            for pool in self.pools.values():
                n_before = len(pool.inflight) + len(pool.gathers)
                got = pool.poll(now)
                results.extend(got)
                if got or len(pool.inflight) + len(pool.gathers) < n_before:
                    progressed = True
            if not progressed:
                pending = [p for p in self.pools.values() if p.inflight or p.gathers]
                if pending:
                    _time.sleep(0.0002)
                elif any(p.active for p in self.pools.values()):
                    continue  # the next iteration launches their slice
                elif i < n:
                    dt = reqs[i].arrival - now()
                    if dt > 0:
                        _time.sleep(min(dt, 0.002))
                elif any(waiting.values()):
                    # nothing runs and the waiting requests do not fit: cannot progress
                    big = [r for q in waiting.values() for r in q][0]
                    raise RuntimeError("request {} needs more lanes ({}) than its pool holds ({})".format(
                        big.rid, big.state.shape[1], self.pools[big.system].C))
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
