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
from .core import Module, lanes_struct
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
        # a module of the pool's own (not the integrators' shared one): its
        # launches run on the pool's streams, and a module's launches must be
        # ordered (its cold-row buffer holds per-launch data)
        self.mod = Module(self.dec, self.order, self.dev.index)
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


def _next_pow2(n):
    r = 1
    while r < n:
        r <<= 1
    return r


class _Ranges:
    """First-fit allocator of contiguous lane ranges (a request's lanes are
    contiguous, so that admitting and gathering it are 2D copies)."""

    def __init__(self, n):
        self.free = [(0, n)]  # sorted (start, length)
        self.n_free = n

    def alloc(self, n):
        for k, (s, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    del self.free[k]
                else:
                    self.free[k] = (s + n, ln - n)
                self.n_free -= n
                return s
        return -1

    def release(self, s, n):
        import bisect

        k = bisect.bisect_left(self.free, (s, 0))
        self.free.insert(k, (s, n))
        # merge with the neighbours
        if k + 1 < len(self.free) and self.free[k][0] + self.free[k][1] == self.free[k + 1][0]:
            self.free[k] = (s, self.free[k][1] + self.free[k + 1][1])
            del self.free[k + 1]
        if k > 0 and self.free[k - 1][0] + self.free[k - 1][1] == self.free[k][0]:
            self.free[k - 1] = (self.free[k - 1][0], self.free[k - 1][1] + self.free[k][1])
            del self.free[k]
        self.n_free += n


@dataclass
class _RActive:
    req: Request
    start: int
    admitted: float
    retiring: bool = False


class ResidentPool:
    """Device lanes of one ODE system served by one resident kernel
    (``hyk_serve``) that takes newly admitted lanes from a device ring while
    it runs, so that a request never waits for a slice boundary or a
    relaunch.

    Admission copies a request's rows (state, parameters, time, final time,
    bookkeeping, owner, status) into a contiguous range of the pool's tables
    and then appends the range's lane indices to the ring and advances its
    tail; retirement reads the per-request finished-lane counters the kernel
    keeps and copies a finished request's range back.  All of it is done by
    stream-ordered copies (``hyk_memcpy2d``) on an I/O stream: the kernel
    holds the pool's share of the SMs, so no other kernel could start.  The
    kernel's waits are bounded: with nothing to do for ``idle_ms`` it returns
    (HYK_SERVE_IDLE) and the pool launches it again with the next admission;
    once any thread has returned, the pool stops the launch (its idle threads
    leave, threads holding lanes finish them) and starts a fresh one, so the
    queue is never served by a thinned-out grid."""

    def __init__(self, name, sys, tol, capacity, device, grid_share=1.0, idle_ms=20.0, max_wait_ms=60000.0,
                 max_requests=1 << 16):
        self.name = name
        self.dec = taylor_decompose(sys)
        self.order = order_from_tol(tol)
        self.dev = torch.device(device)
        # a module of the pool's own (not the integrators' shared one): its
        # launches run on the pool's streams, and a module's launches must be
        # ordered (its cold-row buffer holds per-launch data)
        self.mod = Module(self.dec, self.order, self.dev.index)
        info = self.mod.info_dict()
        if info["team_size"] != 1:
            raise _lib.HykError("the resident serving pool needs a lane-form module")
        self.grid_ctas = max(1, int(info["n_sm"] * info["ctas_per_sm"] * grid_share))
        self.C = int(capacity)
        ne, npar, C = self.dec.n_eq, self.dec.n_pars, self.C
        b = ne + npar
        self.R = {"thi": b, "tlo": b + 1, "tf": b + 2, "rem_hi": b + 3, "rem_lo": b + 4, "min_h": b + 5,
                  "max_h": b + 6, "last_h": b + 7}
        self.RF = b + 8
        f = dict(device=self.dev)
        self.F = torch.zeros((self.RF, C), dtype=torch.float64, **f)
        self.I = torch.zeros((4, C), dtype=torch.int64, **f)  # outcome, n_steps, n_iter, owner
        self.I[3].fill_(-1)
        self.status = torch.full((C,), _DONE, dtype=torch.int32, **f)
        self.ring_cap = _next_pow2(max(C, 2))
        self.ring = torch.zeros(self.ring_cap, dtype=torch.int64, **f)
        # device words: head, tail, inflight (u64); stop, status (u32)
        self.words = torch.zeros(3, dtype=torch.int64, **f)
        self.flags = torch.zeros(2, dtype=torch.int32, **f)
        self.done = torch.zeros(int(max_requests) + 1, dtype=torch.int32, **f)
        self.tail_h = 0
        self.ranges = _Ranges(C)
        self.active: dict = {}
        self.kstream = torch.cuda.Stream(self.dev)
        self.io = torch.cuda.Stream(self.dev)
        self.kernel_ev = None  # completion of the running launch
        self.draining = False
        self.idle_ns = int(idle_ms * 1e6)
        self.max_wait_ns = int(max_wait_ms * 1e6)
        self.lane_steps = 0
        self.keep = deque()  # (event, pinned buffers) alive until their copies are done
        self.poll_ev = None
        self.poll_host = None
        self.gathers: deque = deque()
        self.top_rid = 0

    @property
    def n_free(self):
        return self.ranges.n_free

    def reserve_requests(self, n):
        """Room for request indices below n in the finished-lane counters (a
        running launch is drained first; its counts are carried over)."""
        if n + 1 > self.done.numel():
            if self.kernel_ev is not None:
                self.stop_kernel(wait=True)
            torch.cuda.synchronize(self.dev)
            new = torch.zeros(n + 1, dtype=torch.int32, device=self.dev)
            self._copy(new.data_ptr(), 4, self.done.data_ptr(), 4, self.done.numel() * 4, 1)
            self.io.synchronize()
            self.done = new

    def _copy(self, dst, dpitch, src, spitch, width, height, stream=None):
        L = _lib.load()
        st = self.io if stream is None else stream
        if height == 1:
            dpitch = spitch = width  # one row: the pitches do not matter
        with torch.cuda.device(self.dev):
            _lib.check(L.hyk_memcpy2d(dst, dpitch, src, spitch, width, height,
                                      ctypes.c_void_p(st.cuda_stream)), "hyk_memcpy2d")

    def _free_keep(self):
        while self.keep and self.keep[0][0].query():
            self.keep.popleft()

    def admit(self, reqs, now):
        """Admit the longest prefix of `reqs` whose requests each find a
        contiguous range of free lanes; returns how many were admitted."""
        self._free_keep()
        ne, npar, RF, R, C = self.dec.n_eq, self.dec.n_pars, self.RF, self.R, self.C
        k = 0
        starts = []
        while k < len(reqs):
            st = self.ranges.alloc(reqs[k].state.shape[1])
            if st < 0:
                break
            starts.append(st)
            k += 1
        if k == 0:
            return 0
        self.top_rid = max(self.top_rid, max(r.rid for r in reqs[:k]) + 1)
        self.reserve_requests(self.top_rid)
        bufs = []
        order_h = []
        for r, st in zip(reqs[:k], starts):
            n = r.state.shape[1]
            blk = np.empty((RF, n))
            blk[:ne] = r.state
            if npar:
                blk[ne: ne + npar] = np.asarray(r.pars, dtype=np.float64).reshape(npar, n)
            t0 = np.full(n, float(r.t0))
            tf = np.full(n, float(r.t_final))
            blk[R["thi"]], blk[R["tlo"]], blk[R["tf"]] = t0, 0.0, tf
            # remaining time = tf - t0 in double-length arithmetic (the
            # operations of the propagation initialisation kernel)
            sm = tf - t0
            bb = sm - tf
            e = (tf - (sm - bb)) + (-t0 - bb)
            e = e + 0.0
            hi = sm + e
            lo = e - (hi - sm)
            blk[R["rem_hi"]], blk[R["rem_lo"]] = hi, lo
            blk[R["min_h"]], blk[R["max_h"]], blk[R["last_h"]] = np.inf, 0.0, 0.0
            ints = np.zeros((4, n), dtype=np.int64)
            ints[0] = -4294967299
            ints[3] = r.rid
            stat = np.where((hi == 0) & (lo == 0), _lib.LANE_DONE, 0).astype(np.int32)
            hb = torch.from_numpy(blk).pin_memory()
            hi_ = torch.from_numpy(ints).pin_memory()
            hs = torch.from_numpy(stat).pin_memory()
            bufs += [hb, hi_, hs]
            self._copy(self.F.data_ptr() + st * 8, C * 8, hb.data_ptr(), n * 8, n * 8, RF)
            self._copy(self.I.data_ptr() + st * 8, C * 8, hi_.data_ptr(), n * 8, n * 8, 4)
            self._copy(self.status.data_ptr() + st * 4, C * 4, hs.data_ptr(), n * 4, n * 4, 1)
            order_h.append(np.arange(st, st + n, dtype=np.int64))
            self.active[r.rid] = _RActive(r, st, now)
        # the lane indices into the ring, then the new tail
        lanes = torch.from_numpy(np.concatenate(order_h)).pin_memory()
        bufs.append(lanes)
        m = lanes.numel()
        pos = self.tail_h % self.ring_cap
        first = min(m, self.ring_cap - pos)
        self._copy(self.ring.data_ptr() + pos * 8, 8, lanes.data_ptr(), 8, first * 8, 1)
        if first < m:
            self._copy(self.ring.data_ptr(), 8, lanes.data_ptr() + first * 8, 8, (m - first) * 8, 1)
        self.tail_h += m
        tail = torch.tensor([self.tail_h], dtype=torch.int64).pin_memory()
        bufs.append(tail)
        self._copy(self.words.data_ptr() + 8, 8, tail.data_ptr(), 8, 8, 1)
        ev = torch.cuda.Event()
        ev.record(self.io)
        self.keep.append((ev, bufs))
        self.ensure_kernel()
        return k

    def _launch(self):
        L = _lib.load()
        a = {"rem_hi": self.F[self.R["rem_hi"]], "rem_lo": self.F[self.R["rem_lo"]], "outcome": self.I[0],
             "min_h": self.F[self.R["min_h"]], "max_h": self.F[self.R["max_h"]], "n_steps": self.I[1],
             "n_iter": self.I[2], "last_h": self.F[self.R["last_h"]], "status": self.status}
        d = _lib.hyk_prop_t(
            self.F[self.R["tf"]].data_ptr(), None, None, 0, None, 0, None, None, None, None, 0,
            a["rem_hi"].data_ptr(), a["rem_lo"].data_ptr(), a["outcome"].data_ptr(), a["min_h"].data_ptr(),
            a["max_h"].data_ptr(), a["n_steps"].data_ptr(), a["n_iter"].data_ptr(), None, a["last_h"].data_ptr(),
            None, a["status"].data_ptr(), None, 0, None, None, None, 0, 0,
        )
        ne = self.dec.n_eq
        lanes = lanes_struct(self.F[:ne], self.F[ne: ne + self.dec.n_pars], self.F[self.R["thi"]],
                             self.F[self.R["tlo"]])
        sv = _lib.hyk_serve_t(
            self.ring.data_ptr(), self.ring_cap, self.words.data_ptr(), self.words.data_ptr() + 8,
            self.flags.data_ptr(), self.I[3].data_ptr(), self.done.data_ptr(), self.words.data_ptr() + 16,
            self.flags.data_ptr() + 4, self.idle_ns, self.max_wait_ns, self.grid_ctas,
        )
        # a fresh launch starts with the stop flag and the status word clear
        # (a copy: another pool's launch may hold every other SM)
        zero = torch.zeros(2, dtype=torch.int32).pin_memory()
        self._copy(self.flags.data_ptr(), 8, zero.data_ptr(), 8, 8, 1)
        zev = torch.cuda.Event()
        zev.record(self.io)
        self.keep.append((zev, [zero]))
        with torch.cuda.device(self.dev):
            self.kstream.wait_stream(self.io)
            _lib.check(L.hyk_serve(self.mod.handle, lanes, d, sv, ctypes.c_void_p(self.kstream.cuda_stream)),
                       "hyk_serve")
            ev = torch.cuda.Event()
            ev.record(self.kstream)
        self.kernel_ev = ev
        self.draining = False

    def kernel_running(self):
        return self.kernel_ev is not None and not self.kernel_ev.query()

    def ensure_kernel(self):
        """Launch the kernel unless a launch that still takes work is running."""
        if self.kernel_running() and not self.draining:
            return
        if self.kernel_running():
            return  # a draining launch ends soon; poll() starts the next one
        self._launch()

    def stop_kernel(self, wait=False):
        if self.kernel_ev is None:
            return
        one = torch.ones(1, dtype=torch.int32).pin_memory()
        self._copy(self.flags.data_ptr(), 4, one.data_ptr(), 4, 4, 1)
        ev = torch.cuda.Event()
        ev.record(self.io)
        self.keep.append((ev, [one]))
        self.draining = True
        if wait:
            self.kernel_ev.synchronize()

    def poll(self, now_fn, block=False):
        """Read the finished-lane counters (and the kernel's status word)
        without waiting for the kernel; gather the finished requests; return
        the results whose copies have completed."""
        out = []
        if self.poll_ev is not None and (block or self.poll_ev.query()):
            self.poll_ev.synchronize()
            counts, flags = self.poll_host
            self.poll_ev = None
            cn = counts.numpy()
            done = [rid for rid, a in self.active.items()
                    if not a.retiring and rid < cn.size and cn[rid] >= a.req.state.shape[1]]
            if done:
                self._gather(done)
            if int(flags.numpy()[1]) != 0 and self.kernel_running() and not self.draining:
                self.stop_kernel()  # threads are leaving: end this launch, start a fresh one
        if self.poll_ev is None and self.active:
            n = self.top_rid
            counts = torch.empty(n, dtype=torch.int32).pin_memory()
            flags = torch.empty(2, dtype=torch.int32).pin_memory()
            self._copy(counts.data_ptr(), n * 4, self.done.data_ptr(), n * 4, n * 4, 1)
            self._copy(flags.data_ptr(), 8, self.flags.data_ptr(), 8, 8, 1)
            self.poll_ev = torch.cuda.Event()
            self.poll_ev.record(self.io)
            self.poll_host = (counts, flags)
        if self.kernel_ev is not None and self.kernel_ev.query() and (self.draining or self.tail_pending()):
            if self.tail_pending():
                self._launch()
            else:
                self.draining = False
        while self.gathers and (block or self.gathers[0][0].query()):
            ev, host, acts = self.gathers.popleft()
            ev.synchronize()
            out.extend(self._results(host, acts, now_fn()))
        return out

    def tail_pending(self):
        """Whether admitted lanes may still wait in the ring for a kernel."""
        return any(not a.retiring for a in self.active.values())

    def _gather(self, done):
        acts = [self.active[rid] for rid in done]
        RF, C = self.RF, self.C
        for a in acts:
            a.retiring = True
        host = []
        for a in acts:
            n = a.req.state.shape[1]
            hf = torch.empty((RF, n), dtype=torch.float64).pin_memory()
            hi = torch.empty((3, n), dtype=torch.int64).pin_memory()
            self._copy(hf.data_ptr(), n * 8, self.F.data_ptr() + a.start * 8, C * 8, n * 8, RF)
            self._copy(hi.data_ptr(), n * 8, self.I.data_ptr() + a.start * 8, C * 8, n * 8, 3)
            host.append((hf, hi))
        ev = torch.cuda.Event()
        ev.record(self.io)
        self.gathers.append((ev, host, acts))

    def _results(self, host, acts, t):
        ne, R = self.dec.n_eq, self.R
        out = []
        for (hf, hi), act in zip(host, acts):
            h, ints = hf.numpy(), hi.numpy()
            ns = ints[1].copy()
            out.append(Result(act.req.rid, self.name, h[:ne].copy(), h[R["thi"]].copy(), ints[0].copy(), ns,
                              h[R["min_h"]].copy(), h[R["max_h"]].copy(), arrival=act.req.arrival,
                              admitted=act.admitted, finished=t))
            self.lane_steps += int(ns.sum())
            self.ranges.release(act.start, act.req.state.shape[1])
            del self.active[act.req.rid]
        return out

    def busy(self):
        return bool(self.active or self.gathers)

    # the slice interface of LanePool (the resident kernel needs no slices)
    inflight: deque = deque()

    def depth(self):
        return 0

    def launch_slice(self):
        return False

    def close(self):
        """Stop the kernel (its idle threads return at once) and wait for it.
        The kernel reads the pool's ring and words while it runs, so it must
        end before they are freed: Server.run closes its resident pools when
        the stream is served, and a pool also closes itself when collected."""
        if self.kernel_ev is not None:
            self.stop_kernel(wait=True)
        self.kernel_ev = None
        self.io.synchronize()

    def __del__(self):
        try:
            if self.__dict__.get("kernel_ev") is not None:
                self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


class Server:
    """Continuous-batching server over a set of ODE systems.

    ``systems``: name -> (sys, tol).  ``hbm_budget``: bytes of lane state per
    system pool (admission by footprint).  ``mode``: "slice" (the default:
    time slices of the persistent kernel over every admitted lane, relaunched
    by the host, LanePool) or "resident" (one resident kernel per system on
    an equal share of the SMs, fed from a device ring, ResidentPool: the
    lower latency while the GPU is lightly loaded, but its threads serve the
    ring in order, so under load short requests wait behind long ones).
    ``slice_iters``: the most steps per lane in one slice; ``quantum_ms``:
    the target duration of a slice."""

    def __init__(self, systems, hbm_budget=2 << 30, slice_iters=1024, device="cuda:0", max_lanes=1 << 21,
                 quantum_ms=2.0, mode="slice"):
        if mode not in ("resident", "slice"):
            raise ValueError("mode must be 'resident' or 'slice'")
        self.pools = {}
        self.mode = mode
        for name, (sys, tol) in systems.items():
            dec = taylor_decompose(sys)
            bpl = (dec.n_eq + dec.n_pars + 16) * 8
            cap = int(min(max_lanes, hbm_budget // bpl))  # lanes that fit the pool's HBM budget
            pool = None
            if mode == "resident":
                # one resident kernel per system, each on an equal share of the SMs
                try:
                    pool = ResidentPool(name, sys, tol, cap, device, grid_share=1.0 / len(systems))
                except _lib.HykError:
                    pool = None  # a team-form system: time slices
            self.pools[name] = pool or LanePool(name, sys, tol, cap, device, slice_iters, quantum_ms * 1e-3)
        self._warm = False

    def warm(self):
        """Serve one zero-duration request per pool through the whole path
        (admission, a launch, counting, retirement): the first launch of each
        pool pays one-time costs (seconds for the first slice of a pool on a
        fresh process: module loading and the first use of its host and device
        buffers) that would otherwise fall on the first real requests.  Done by
        the first run() unless called before."""
        if self._warm:
            return
        self._warm = True
        dummies = []
        for i, (name, pool) in enumerate(self.pools.items()):
            st = np.zeros((pool.dec.n_eq, 1))
            pa = np.zeros((pool.dec.n_pars, 1)) if pool.dec.n_pars else None
            dummies.append(Request(name, st, 0.0, pars=pa, rid=i))
        self.run(dummies, realtime=False)

    def run(self, requests, realtime=True):
        """Serve `requests` (with arrival times in seconds); returns the results
        in completion order.  With ``realtime`` the arrivals follow the wall
        clock; otherwise each request is available from the start."""
        self.warm()
        reqs = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(reqs):
            if r.rid < 0:
                r.rid = i
        top = max((r.rid for r in reqs), default=0) + 1
        for p in self.pools.values():
            p.reserve_requests(top)
            if isinstance(p, ResidentPool):
                # the finished-lane counters are per request index: a new run
                # may reuse the indices of an earlier one (no kernel runs now)
                torch.cuda.synchronize(p.dev)
                p.done.zero_()
                torch.cuda.synchronize(p.dev)
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
        self.close()
        return results

    def close(self):
        """End every resident kernel (none outlives a run)."""
        for p in self.pools.values():
            if isinstance(p, ResidentPool):
                p.close()

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
