"""Benchmark: FP64 Taylor trajectory-steps/s on the 2^20-orbit Kepler ensemble.

Workload (the reference metric's configuration): 3D Keplerian two-body, mu = 1,
tol = 1e-15 (Taylor order 19), 2^20 orbits with a ~ U[0.5, 2], e ~ U[0, 0.6],
i ~ U[0, pi/4], Omega, omega, M ~ U[0, 2 pi) (seeded synthetic elements
converted to Cartesian), propagated from t = 0 to t = 200.  One bench "step"
propagates the whole ensemble over 200 / K time units, so the K timed steps
together are exactly the propagation to t = 200.  The ensemble stays resident
in HBM; its per-lane state and bookkeeping (~170 MB) exceed the 129 MB L2.

value: trajectory-steps/s (sum over lanes of accepted non-zero steps / time)
of the persistent batched kernel.  e2e: the same metric through the public
API with the state copied from pinned host memory before, and the state and
step counts copied back after, every step.  paths.plain: the one-launch-per-
step form over the unfinished lanes (listed before each launch);
paths.plain_inplace: one launch per step over every lane (the naive drop-in
form).  roofline: algorithmic FP64 flops of the propagation kernel (the
measurement contract's count, contract_flops; the code generator's smaller
count beside it as flops_per_traj_step_generated / frac_generated) / its
CUDA-event duration, against the FP64 FMA peak measured in the same process.  cpu_baseline: the compiled CPU stepper that
stands in for the reference's compiled batch stepper (generated recurrences in
the reference's arithmetic, g++ -O3, vector batches of lanes, OpenMP over all
host cores; oracle/cpu_batch.py) on a bounded sample of the same orbits.

--impl reference times that compiled CPU stepper alone (the reference itself,
heyoka.py over the heyoka C++ library, is not installable here).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "heyoka.py_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "FP64 Taylor trajectory-steps/s, 2^20-orbit Kepler ensemble (tol 1e-15, t=0..200)"
UNIT = "trajectory-steps/s"
T_END = 200.0
TOL = 1e-15

# DRAM traffic of one persistent Kepler launch per lane, from ncu
# (dram__bytes_read.sum + dram__bytes_write.sum = 18.55 MB + 1.65 MB for 2^17 orbits).
KEPLER_DRAM_BYTES_PER_LANE = (18.546e6 + 1.652e6) / 131072

def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="hyk", choices=["hyk", "reference"])
    ap.add_argument("--orbits", type=int, default=1 << 20)
    ap.add_argument("--cpu-sample", type=int, default=32768)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="kepler", choices=["kepler", "kepler-f32", "serve", "pendulum", "cr3bp-adjoint", "oss", "forms",
                             "occupancy", "plain"],
                    help="kepler: the headline metric; serve: the Poisson request stream (p50/p99 latency); "
                         "pendulum: 4096 trajectories through ensemble_propagate_until; "
                         "cr3bp-adjoint: 65536 trajectories forward plus discrete adjoint")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: requests per second")
    ap.add_argument("--duration", type=float, default=10.0, help="serve: seconds of arrivals")
    ap.add_argument("--slice", type=int, default=1024, help="serve: the most steps per lane in one slice")
    ap.add_argument("--quantum-ms", type=float, default=2.0, help="serve: target duration of a slice")
    ap.add_argument("--serve-mode", default="slice", choices=["resident", "slice"],
                    help="serve: time slices relaunched by the host (default), or resident kernels fed from a "
                         "device ring")
    ap.add_argument("--members", type=int, default=65536, help="oss, cr3bp-adjoint: trajectories")
    ap.add_argument("--autotune", action="store_true",
                    help="oss: pick the kernel configuration by measurement (hyk.autotune, cached per system)")
    ap.add_argument("--team-size", type=int, default=0,
                    help="threads per trajectory (0: chosen per system, 1: lane form, 2..32: team form)")
    return ap.parse_args()


def dist_init(n):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    return rank, world


_ICS = {}


def _ensemble_ics(seed):
    from hyk import workloads as W

    if seed not in _ICS:
        _ICS[seed] = W.kepler_ics(1 << 20, seed=seed)
    return _ICS[seed]


def contract_flops(sys_, order):
    """Algorithmic FP64 flops of one trajectory-step under the measurement
    contract of the hot-path plan: F = sum over the decomposition's operations
    of sum_{n=0}^{p} cost(n) + N p (state coefficients) + 2 N p (Horner) +
    2 N + 30 (step size), with per-order costs add/sub/neg and products or
    quotients by a number or parameter 1, mul 2n+1, square n+2, div 2n+2,
    sqrt n+3, pow 4n+3, exp 2n+1, log 2n+3, a sin/cos pair 4n+2 (a lone sin or
    cos counted as the pair) plus p once for its j a_j."""
    from hyk import decompose as D

    dec = D.taylor_decompose(sys_)
    p, N = int(order), dec.n_eq
    cost = {D.OP_MUL: lambda n: 2 * n + 1, D.OP_SQUARE: lambda n: n + 2, D.OP_DIV: lambda n: 2 * n + 2,
            D.OP_SQRT: lambda n: n + 3, D.OP_POW: lambda n: 4 * n + 3, D.OP_EXP: lambda n: 2 * n + 1,
            D.OP_LOG: lambda n: 2 * n + 3}
    F = 0
    trig = set()
    for op, aux, a, b in dec.ops:
        consts = (D.ARG_NUM, D.ARG_PAR)
        if op in (D.OP_ADD, D.OP_SUB, D.OP_NEG) or (op in (D.OP_MUL, D.OP_DIV) and (a[0] in consts or b[0] in consts)):
            F += p + 1
        elif op in (D.OP_SIN, D.OP_COS):
            if a in trig:  # the other half of a pair already counted
                continue
            trig.add(a)
            F += sum(4 * n + 2 for n in range(p + 1)) + p
        else:
            F += sum(cost[op](n) for n in range(p + 1))
    return F + N * p + 2 * N * p + 2 * N + 30


_CPU = {}


def cpu_stepper_setup(sys_, order, probe_state, probe_t):
    """The compiled CPU stepper's batch width (2 or 4 lanes, whichever runs the probe faster on these cores)
    and the host cores' measured FP64 FMA peak."""
    import cpu_batch

    key = (id(sys_), order)
    if key not in _CPU:
        best = None
        for b in (2, 4):
            cpu_batch.ensemble_until(sys_, probe_state, None, 0.0, 0.1 * probe_t, order=order, batch=b)
            t0 = time.perf_counter()
            r = cpu_batch.ensemble_until(sys_, probe_state, None, 0.0, probe_t, order=order, batch=b)
            v = float(r["n_steps"].sum()) / (time.perf_counter() - t0)
            if best is None or v > best[1]:
                best = (b, v)
        _CPU[key] = {"batch": best[0], "peak": cpu_batch.fp64_peak(0, 1.0)}
    return _CPU[key]


def cpu_baseline(n_orbits, seed, t_end, steps=1):
    """Time the compiled CPU stepper (the stand-in for the reference's compiled batch stepper) on n_orbits of
    the same ensemble, all host threads; the oracle's interpreter on a small sample as a secondary figure."""
    import numpy as np

    import cpu_batch
    import pyoracle
    from hyk import workloads as W

    st = _ensemble_ics(seed)
    idx = np.random.default_rng(123).choice(st.shape[1], n_orbits, replace=False)
    sample = np.ascontiguousarray(st[:, np.sort(idx)])
    sys_ = W.kepler_sys()
    setup = cpu_stepper_setup(sys_, 19, sample[:, :512], t_end)
    fl = contract_flops(sys_, 19)
    best = None
    tot_steps = 0
    threads = 0
    for _ in range(steps):
        t0 = time.perf_counter()
        r = cpu_batch.ensemble_until(sys_, sample, None, 0.0, t_end, order=19, batch=setup["batch"])
        dt = time.perf_counter() - t0
        tot_steps, threads = int(r["n_steps"].sum()), r["threads"]
        v = tot_steps / dt
        best = v if best is None else max(best, v)
    # secondary: the oracle's per-operation interpreter (the round-1 baseline), 1024 orbits
    isample = np.ascontiguousarray(sample[:, :1024])
    t0 = time.perf_counter()
    ri = pyoracle.ensemble_until(sys_, isample, None, 0.0, t_end, order=19, batch=8, n_threads=threads, mode=0)
    interp = float(ri["n_steps"].sum()) / (time.perf_counter() - t0)
    return {
        "value": best,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": "{} of the 2^20 orbits (seeded subset), t=0..{:g}, {} trajectory-steps: generated recurrences in the "
                  "reference's arithmetic compiled with g++ -O3, batches of {} lanes (vector types), OpenMP over {} host "
                  "threads (oracle/cpu_batch.py)".format(n_orbits, t_end, tot_steps, setup["batch"], threads),
        "gflops": best * fl / 1e9,
        "host_fp64_peak_gflops": setup["peak"] / 1e9,
        "frac_of_host_peak": best * fl / setup["peak"],
        "flops_per_traj_step": fl,
        "interpreter": {"value": interp, "sample": "1024 orbits, the oracle's per-operation interpreter (pyoracle), "
                                                   "batches of 8, {} threads".format(threads)},
    }


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = (
        "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
        "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
        "clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index):
        self.p = None
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def parity_checks(dev, K):
    """Parity at the headline configuration (untimed): 1024 seeded orbits of the
    ensemble propagated by the GPU with the bench's own schedule (K calls of
    200 / K time units), against the oracle in the reference's arithmetic on
    the same schedule (final-state relative error, step-count agreement) and
    against the binary128 states of tests/golden/kepler_t200_quad_1024.npz (the
    error of each arithmetic at t = 200)."""
    import numpy as np

    import hyk
    import pyoracle
    from hyk import workloads as W

    fx = np.load(os.path.join(ROOT, "tests", "golden", "kepler_t200_quad_1024.npz"))
    st = np.ascontiguousarray(_ensemble_ics(1)[:, fx["idx"]])
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=TOL, device="cuda:{}".format(dev))
    ref = pyoracle.Oracle(W.kepler_sys(), st, order=ta.order, mode=0)
    steps_gpu = np.zeros(st.shape[1], dtype=np.int64)
    steps_ref = np.zeros(st.shape[1], dtype=np.int64)
    for k in range(K):
        t = (k + 1) * (T_END / K)
        ta.propagate_until(t)
        r = ref.propagate_until(t)
        steps_gpu += ta.propagate_res_tensors["n_steps"].cpu().numpy()
        steps_ref += r["n_steps"].astype(np.int64)
    g = np.asarray(ta.state)

    def rel(a, b):
        return np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)

    e_ref = rel(g, ref.state)
    q = fx["state_t200"]
    eg, er = rel(g, q), rel(ref.state, q)
    return {
        "orbits": int(st.shape[1]),
        "vs_reference_arithmetic": {"max_rel_err": float(e_ref.max()), "median_rel_err": float(np.median(e_ref)),
                                    "frac_le_1e-12": float(np.mean(e_ref <= 1e-12)),
                                    "step_count_agreement": float(np.mean(steps_gpu == steps_ref))},
        "vs_binary128": {"gpu_max": float(eg.max()), "gpu_median": float(np.median(eg)),
                         "gpu_p99": float(np.quantile(eg, 0.99)),
                         "reference_arithmetic_max": float(er.max()), "reference_arithmetic_median": float(np.median(er)),
                         "reference_arithmetic_p99": float(np.quantile(er, 0.99))},
        "note": "the reference arithmetic is itself farther than 1e-12 from the binary128 solution on some orbits "
                "at t = 200; the GPU's error distribution against binary128 is the comparison that holds there",
    }


def run_reference(args, rank, world):
    if rank != 0:
        return
    t0 = time.perf_counter()
    for _ in range(args.warmup):
        cpu_baseline(min(args.cpu_sample, 1024), 1, T_END)
    vals = []
    last = None
    t_start = time.perf_counter()
    for _ in range(args.steps):
        last = cpu_baseline(args.cpu_sample, 1, T_END)
        vals.append(last["value"])
    wall = time.perf_counter() - t_start
    v = statistics.median(vals)
    cb = dict(last)
    cb["value"] = v
    line = {
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Kepler elements)",
        "config": {"workload": "kepler-2^20 tol=1e-15 t=0..200 (CPU sample of {} orbits per step)".format(args.cpu_sample)},
        "impl": "reference",
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "heyoka.py needs the heyoka C++ library, which is not installable offline; the timed CPU code stands in "
                "for its compiled batch stepper: this repository's generated recurrences in the reference's arithmetic, "
                "compiled with g++ -O3 over vector batches, and the oracle's restatement of the batch propagate loop "
                "(oracle/cpu_batch.py, oracle/hyk_cpu_batch.cpp), bit-identical to the oracle's reference arithmetic",
        "wall_s": time.perf_counter() - t0,
    }
    print(json.dumps(line), flush=True)


def serve_stream(rate, duration, seed=4):
    """Poisson arrivals; size ~ round(logU[1, 4096]); system ~ U{pendulum, kepler,
    cr3bp} with the workload initial-condition laws; horizon ~ logU[1, 1000]."""
    import math

    import numpy as np

    from hyk import serve
    from hyk import workloads as W

    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        size = int(round(math.exp(rng.uniform(0.0, math.log(4096.0)))))
        kind = ["pendulum", "kepler", "cr3bp"][int(rng.integers(3))]
        tf = float(math.exp(rng.uniform(0.0, math.log(1000.0))))
        s = int(rng.integers(1 << 30))
        if kind == "pendulum":
            st, pa = W.pendulum_ics(size, seed=s), None
        elif kind == "kepler":
            st, pa = W.kepler_ics(size, seed=s), None
        else:
            st, pa = W.cr3bp_ics(size, seed=s)
        reqs.append(serve.Request(kind, st, tf, pars=pa, arrival=t, rid=len(reqs)))
    return reqs


def run_serve(args):
    import numpy as np
    import torch

    import hyk
    from hyk import serve
    from hyk import workloads as W

    systems = {"pendulum": (W.pendulum_sys(), 1e-15), "kepler": (W.kepler_sys(), 1e-15), "cr3bp": (W.cr3bp_sys(), 1e-15)}
    reqs = serve_stream(args.rate, args.duration)
    srv = serve.Server(systems, hbm_budget=4 << 30, slice_iters=args.slice, quantum_ms=args.quantum_ms,
                       mode=args.serve_mode)
    srv.run(serve_stream(50.0, 0.2, seed=99), realtime=False)  # warm-up: compile, first launches
    for p in srv.pools.values():
        p.lane_steps = 0
    clk = Clocks(0)
    t0 = time.perf_counter()
    res = srv.run(reqs, realtime=True)
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    stats = serve.latency_stats(res)
    steps = srv.trajectory_steps()
    # isolated solve time of a sample of the same requests (alone on the GPU)
    rng = np.random.default_rng(5)
    sample = rng.choice(len(reqs), size=min(200, len(reqs)), replace=False)
    by_id = {r.rid: r for r in res}
    ratios, iso = [], []
    for i in sample:
        r = reqs[int(i)]
        sys_, tol = systems[r.system]
        ta = hyk.taylor_adaptive_batch(sys_, r.state, pars=r.pars, tol=tol)
        torch.cuda.synchronize()
        a = time.perf_counter()
        ta.propagate_until(r.t_final)
        ta.state.cpu()
        b = time.perf_counter()
        iso.append(b - a)
        ratios.append(by_id[r.rid].latency / (b - a))
    line = {
        "metric": "serving: FP64 trajectory-steps/s and p50/p99 request latency, Poisson stream",
        "value": steps / wall,
        "unit": UNIT,
        "n_gpus": 1,
        "higher_is_better": True,
        "dtype": "f64",
        "data": "synthetic (seeded request stream)",
        "config": {
            "workload": "serve: Poisson {:g} req/s for {:g} s, size round(logU[1,4096]), system U{{pendulum,kepler,cr3bp}}, "
                        "horizon logU[1,1000], tol 1e-15".format(args.rate, args.duration),
            "requests": len(reqs),
            "mode": args.serve_mode,
            "slice_iters_max": args.slice,
            "quantum_ms": args.quantum_ms,
            "pool_capacity": {k: p.C for k, p in srv.pools.items()},
        },
        "latency": stats,
        "isolated_solve_ms": {"p50": float(np.percentile(iso, 50) * 1e3), "p99": float(np.percentile(iso, 99) * 1e3)},
        "latency_over_isolated": {"p50": float(np.percentile(ratios, 50)), "p99": float(np.percentile(ratios, 99))},
        "offered_traj_per_s": sum(r.state.shape[1] for r in reqs) / args.duration,
        "wall_s": wall,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_pendulum(args):
    """4096 pendulum trajectories (1024 ensemble iterations x batch 4), tol
    2.2e-16 (order 20), t = 0..100, through ensemble_propagate_until."""
    import numpy as np
    import torch

    import hyk
    import pyoracle
    from hyk import workloads as W

    st = W.pendulum_ics(4096, seed=0)
    ta = hyk.taylor_adaptive_batch(W.pendulum_sys(), np.zeros((2, 4)), tol=2.2e-16)

    def gen(t, i):
        t.set_time(0.0)
        t.state[:] = st[:, 4 * i: 4 * i + 4]
        return t

    hyk.ensemble_propagate_until(ta, 1.0, 1024, gen)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ret = hyk.ensemble_propagate_until(ta, 100.0, 1024, gen)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    steps = sum(sum(r[3] for r in x[0].propagate_res) for x in ret)
    # the same 4096 trajectories as one device batch (no generator calls, no
    # per-iteration integrators): the device's share of the ensemble call
    tb = hyk.taylor_adaptive_batch(W.pendulum_sys(), st, tol=2.2e-16)
    tb.propagate_until(1.0)
    tb.set_time(0.0)
    tb.state[:] = st
    torch.cuda.synchronize()
    b0 = time.perf_counter()
    tb.propagate_until(100.0)
    torch.cuda.synchronize()
    bwall = time.perf_counter() - b0
    bsteps = int(tb.propagate_res_tensors["n_steps"].sum().item())
    import cpu_batch

    csetup = cpu_stepper_setup(W.pendulum_sys(), 20, st[:, :512], 10.0)
    c0 = time.perf_counter()
    cr = cpu_batch.ensemble_until(W.pendulum_sys(), st, None, 0.0, 100.0, order=20, batch=csetup["batch"])
    cwall = time.perf_counter() - c0
    threads = cr["threads"]
    line = {
        "metric": "FP64 Taylor trajectory-steps/s, pendulum ensemble (4096 trajectories, tol 2.2e-16, t=0..100)",
        "value": steps / wall, "unit": UNIT, "n_gpus": 1, "higher_is_better": True, "dtype": "f64",
        "data": "synthetic (x0 ~ U[-1.5,1.5], v0 ~ U[-0.5,0.5], seed 0)",
        "config": {"workload": "pendulum-4096 via ensemble_propagate_until (1024 x batch 4), order 20",
                   "note": "end to end through the public ensemble API: host generator calls, one device batch, "
                           "per-iteration integrators returned"},
        "trajectory_steps": int(steps), "wall_s": wall,
        "paths": {"ensemble_api": steps / wall, "one_device_batch": bsteps / bwall,
                  "note": "the ensemble call's wall time is mostly its 1024 host generator calls and the 1024 "
                          "per-iteration integrators it returns; one_device_batch propagates the same 4096 "
                          "trajectories as one taylor_adaptive_batch"},
        "cpu_baseline": {"value": float(cr["n_steps"].sum()) / cwall, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "the same 4096 trajectories as one batch (no generator calls), compiled CPU "
                                   "stepper (reference arithmetic, batches of {} lanes, oracle/cpu_batch.py)"
                                   .format(csetup["batch"])},
    }
    print(json.dumps(line), flush=True)


def run_cr3bp_adjoint(args):
    """65536 CR3BP trajectories near L4 (mu ~ U[0.005, 0.02] per lane), tol
    1e-15, t = 0..50: forward with the checkpoint tape, then the discrete
    adjoint of loss = sum |r(50) - r*|^2 with respect to the initial state
    and mu."""
    import numpy as np
    import torch

    from hyk import adjoint
    from hyk import workloads as W

    n = args.members
    st, mu = W.cr3bp_ics(n, seed=3)
    rng = np.random.default_rng(3)
    target = torch.tensor(st[:3] + rng.normal(0.0, 1e-2, (3, n)), device="cuda")
    x = torch.tensor(st, device="cuda", requires_grad=True)
    p = torch.tensor(mu, device="cuda", requires_grad=True)
    # warm-up: the whole workload once (compiles both modules, sizes the tape,
    # loads every kernel the timed call uses)
    for _ in range(max(1, args.warmup)):
        xf, _ = adjoint.taylor_flow(W.cr3bp_sys(), x, 50.0, pars=p, tol=1e-15)
        ((xf[:3] - target) ** 2).sum().backward()
        x.grad = None
        p.grad = None
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    xf, _ = adjoint.taylor_flow(W.cr3bp_sys(), x, 50.0, pars=p, tol=1e-15)
    loss = ((xf[:3] - target) ** 2).sum()
    e1.record()
    loss.backward()
    e2.record()
    torch.cuda.synchronize()
    fwd, bwd = e0.elapsed_time(e1) / 1e3, e1.elapsed_time(e2) / 1e3
    line = {
        "metric": "CR3BP forward + discrete adjoint, {} trajectories, tol 1e-15, t=0..50".format(n),
        "value": None, "unit": "s", "n_gpus": 1, "higher_is_better": False, "dtype": "f64",
        "data": "synthetic (states near L4, seed 3)",
        "forward_s": fwd, "backward_s": bwd,
        "grad_finite": bool(torch.isfinite(x.grad).all() and torch.isfinite(p.grad).all()),
        "config": {"workload": "cr3bp-{} forward + adjoint".format(n)},
    }
    line["value"] = fwd + bwd
    print(json.dumps(line), flush=True)


def run_oss(args):
    """Outer-solar-system 6-body ensemble: 65536 members, tol 1e-15 (order
    19), end times log-uniform in [1e3, 1e5] days, propagate_grid over 100
    points per member.  value: the device-resident call (grid and state in
    HBM, output left on the device); kernel: the propagation launch alone
    (CUDA events on its stream); e2e: the public propagate_grid with the
    state and grid copied in from pinned host memory and the (100, 36,
    65536) output copied back to the host."""
    import numpy as np
    import torch

    import hyk
    import pyoracle
    from hyk import workloads as W

    n = args.members
    st, t_end = W.oss_ics(n, seed=2)
    grid = np.linspace(0.0, 1.0, 100).reshape(-1, 1) * t_end.reshape(1, -1)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, team_size=args.team_size)
    gd = torch.tensor(grid, device="cuda")
    tuned = None
    if args.autotune:
        # the kernel configuration measured on this very call (hyk.autotune.tune_call)
        from hyk import autotune

        t_tune = time.perf_counter()
        tuned = autotune.tune_call(ta, lambda t: t.propagate_grid_tensor(gd))
        tuned["tune_s"] = time.perf_counter() - t_tune
    sd = torch.tensor(st, device="cuda")
    g_host = torch.tensor(grid).pin_memory()
    s_host = torch.tensor(st).pin_memory()
    for _ in range(max(3, args.warmup)):
        ta.set_time(0.0)
        ta.state[:] = sd
        ta.propagate_grid_tensor(gd * 1e-2)
    times, ktimes, e2e = [], [], []
    mon = Clocks(0)
    for _ in range(max(1, args.steps)):
        ta.set_time(0.0)
        ta.state[:] = sd
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        ta._launch_events = kev
        e0.record()
        out = ta.propagate_grid_tensor(gd)
        e1.record()
        torch.cuda.synchronize()
        ta._launch_events = None
        times.append(e0.elapsed_time(e1) / 1e3)
        ktimes.append(kev[0].elapsed_time(kev[1]) / 1e3)
    steps = int(ta.propagate_res_tensors["n_steps"].sum().item())
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        ta.set_time(0.0)
        ta.state[:] = s_host.to("cuda", non_blocking=True)
        _, out_np = ta.propagate_grid(g_host.to("cuda", non_blocking=True))
        e2e.append(time.perf_counter() - w0)
    clocks = mon.stop()
    info = ta.module_info
    t_dev, t_k, t_e2e = float(np.median(times)), float(np.median(ktimes)), float(np.median(e2e))
    # CPU baseline: the compiled CPU stepper on 4096 members (evenly spaced), each to its end time, all host
    # threads (propagate_until: the grid's 100 dense outputs, ~3 % of the work, are left out).
    import cpu_batch

    pick = np.linspace(0, n - 1, 4096).astype(np.int64)
    csetup = cpu_stepper_setup(W.oss_sys(), ta.order, np.ascontiguousarray(st[:, pick[:256]]), 1e3)
    c0 = time.perf_counter()
    r = cpu_batch.ensemble_until(W.oss_sys(), np.ascontiguousarray(st[:, pick]), None, 0.0, t_end[pick], order=ta.order,
                                 batch=csetup["batch"])
    cwall = time.perf_counter() - c0
    F = contract_flops(W.oss_sys(), ta.order)
    fl = F * steps / t_k
    peak = hyk.fp64_peak(0, 300.0)
    h2d = st.nbytes + grid.nbytes
    line = {
        "metric": "FP64 Taylor trajectory-steps/s, outer-solar-system 6-body ensemble (65536 members, tol 1e-15, "
                  "propagate_grid 100 points, end times log-uniform [1e3,1e5] days)",
        "value": steps / t_dev, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "higher_is_better": True,
        "dtype": "f64", "data": "synthetic (near-circular orbits, 1e-6 relative Gaussian perturbations, seed 2)",
        "config": {"workload": "oss-6body-{} propagate_grid".format(n), "order": ta.order,
                   "threads_per_trajectory": info["team_size"],
                   "jets": "global memory" if info["smem_per_lane"] == 0 else "shared memory",
                   "block_threads": info["block_lanes"], "ctas_per_sm": info["ctas_per_sm"],
                   "autotune": None if tuned is None else {"best": tuned["best"], "tune_s": tuned["tune_s"],
                                                              "trials": [{k: v for k, v in t.items()
                                                                          if k in ("team", "jets", "block",
                                                                                   "seconds", "skipped")}
                                                                         for t in tuned["trials"]]},
                   "l2": "inputs and the 1.9 GB output exceed L2"},
        "trajectory_steps": steps, "device_s": t_dev, "kernel_s": t_k,
        "e2e": {"value": steps / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(out_np.nbytes)},
        "roofline": {"bound": "fp64", "achieved": fl / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": fl / peak, "traffic": None, "flops_per_traj_step": F,
                     "flops_per_traj_step_generated": info["flops_per_step"],
                     "frac_generated": info["flops_per_step"] * steps / t_k / peak,
                     "note": "contract flops per step x trajectory-steps / propagation-kernel time; peak = in-process "
                             "FP64 FMA probe, of measured (MEASURED_PEAKS.json has no FP64 entry)"},
        "cpu_baseline": {"value": float(r["n_steps"].sum()) / cwall, "unit": UNIT, "cores": r["threads"], "kind": "port",
                         "sample": "4096 of the 65536 members (evenly spaced), propagate_until each member's end time, "
                                   "compiled CPU stepper (reference arithmetic, batches of {} lanes, oracle/cpu_batch.py)"
                                   .format(csetup["batch"]),
                         "gflops": float(r["n_steps"].sum()) / cwall * F / 1e9,
                         "frac_of_host_peak": float(r["n_steps"].sum()) / cwall * F / csetup["peak"]},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_kepler_f32(args):
    """The Kepler ensemble in single precision (fp_type=numpy.float32, tol
    2^-23, order 9): 2^20 orbits propagated over t = 0..200 on the device in
    K steps, as the double headline.  value: device-resident persistent
    propagation; e2e: the public API with pinned float32 host buffers copied in
    and out every step; roofline against the in-process FP32 FMA probe."""
    import numpy as np
    import torch

    import hyk
    import pyoracle
    from hyk import workloads as W

    f32 = np.float32
    K, Wm = max(1, args.steps), max(3, args.warmup)
    dt = T_END / K
    n = args.orbits
    st = W.kepler_ics(n, seed=1).astype(f32)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, fp_type=f32)
    info = ta.module_info
    wcopy = hyk.taylor_adaptive_batch(W.kepler_sys(), st, fp_type=f32)
    for k in range(Wm):
        wcopy.propagate_until((k + 1) * dt)
    del wcopy
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    kevs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    steps_per = []
    clk = Clocks(0)
    torch.cuda.synchronize()
    for k in range(K):
        evs[k][0].record(stream)
        ta._launch_events = kevs[k]
        ta.propagate_until((k + 1) * dt)
        evs[k][1].record(stream)
        steps_per.append(ta.propagate_res_tensors["n_steps"].sum())
    torch.cuda.synchronize()
    clocks = clk.stop()
    ta._launch_events = None
    t_gpu = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    t_k = sum(a.elapsed_time(b) for a, b in kevs) / 1e3
    n_steps = int(torch.stack(steps_per).sum().item())
    ok = bool((ta.propagate_res_tensors["outcome"] == int(hyk.taylor_outcome.time_limit)).all())
    final_t_ok = bool(np.all(ta.time == f32(T_END)))
    # e2e through the public API, float32 host buffers
    host_state = torch.tensor(st).pin_memory()
    out_state = torch.empty_like(host_state).pin_memory()
    out_steps = torch.empty(n, dtype=torch.int64).pin_memory()
    ta2 = hyk.taylor_adaptive_batch(W.kepler_sys(), st, fp_type=f32)
    ta2.propagate_until(dt)
    ta2.set_time(0.0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    cur, e2e_steps = host_state, []
    for k in range(K):
        ta2.state.copy_(cur, non_blocking=True)
        ta2.propagate_until((k + 1) * dt)
        out_state.copy_(ta2.state, non_blocking=True)
        out_steps.copy_(ta2.propagate_res_tensors["n_steps"], non_blocking=True)
        e2e_steps.append(ta2.propagate_res_tensors["n_steps"].sum())
        cur = out_state
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_total = int(torch.stack(e2e_steps).sum().item())
    e2e = {"value": e2e_total / (e0.elapsed_time(e1) / 1e3), "unit": UNIT,
           "h2d_bytes_per_step": int(host_state.numel() * 4),
           "d2h_bytes_per_step": int(out_state.numel() * 4 + out_steps.numel() * 8)}
    del ta2
    # accuracy against the double integrator on a sample of the same orbits
    pick = np.linspace(0, n - 1, 4096).astype(np.int64)
    tdd = hyk.taylor_adaptive_batch(W.kepler_sys(), st[:, pick].astype(np.float64), tol=TOL)
    tdd.propagate_until(T_END)
    err = float(np.max(np.abs(np.asarray(ta.state)[:, pick].astype(np.float64) - np.asarray(tdd.state))))
    del tdd
    peak = hyk.fp32_peak(0, 300.0)
    F = contract_flops(W.kepler_sys(), ta.order)
    fl = F * n_steps / t_k
    cpu = None
    if not args.no_cpu:
        idx = np.random.default_rng(123).choice(n, args.cpu_sample, replace=False)
        sample = np.ascontiguousarray(st[:, np.sort(idx)]).astype(np.float64)
        threads = pyoracle.lib().hyko_max_threads()
        c0 = time.perf_counter()
        r = pyoracle.ensemble_until(W.kepler_sys(), sample, None, 0.0, T_END, order=ta.order, batch=8,
                                    n_threads=threads, mode=0, prec=2)
        cw = time.perf_counter() - c0
        cpu = {"value": float(r["n_steps"].sum()) / cw, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "{} of the 2^20 orbits (seeded subset), t=0..{:g}, float, batches of 8 lanes".format(
                   args.cpu_sample, T_END)}
    line = {
        "metric": "FP32 Taylor trajectory-steps/s, 2^20-orbit Kepler ensemble (fp_type float32, tol 2^-23, t=0..200)",
        "value": n_steps / t_gpu, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": Wm,
        "ms_per_step": t_gpu / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Kepler elements, rounded to float)",
        "config": {"workload": "kepler-2^20 float32 t=0..200", "order": ta.order,
                   "block_lanes": info["block_lanes"], "smem_per_lane": info["smem_per_lane"],
                   "regs_per_thread": info["regs_per_thread"], "ctas_per_sm": info["ctas_per_sm"],
                   "l2": "inputs larger than L2 (state + bookkeeping ~{:.0f} MB)".format(n * 21 * 4 / 1e6)},
        "trajectory_steps": n_steps, "device_s": t_gpu, "kernel_s": t_k, "e2e": e2e,
        # per step: bookkeeping init, the one-step estimate of the longest-first order, the propagation
        "gpu_launches": 3 * K,
        "roofline": {"bound": "fp32", "achieved": fl / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": fl / peak, "traffic": None, "kernel": "hyk_prop_kernel (persistent, float)",
                     "flops_per_traj_step": F, "flops_per_traj_step_generated": info["flops_per_step"],
                     "frac_generated": info["flops_per_step"] * n_steps / t_k / peak,
                     "peak_source": "measured in-process FP32 FMA probe (hyk_fp32_peak), of measured"},
        "cpu_baseline": cpu, "clocks": clocks,
        "checks": {"all_time_limit": ok, "final_time_exact": final_t_ok,
                   "max_abs_diff_vs_double_4096_sample": err},
    }
    print(json.dumps(line), flush=True)


def run_forms(args):
    """Lane form against team form (threads per trajectory) on three systems:
    propagate_until of 65536 outer-solar-system members to t = 2e4 days,
    65536 CR3BP trajectories to t = 50 and 262144 Kepler orbits to t = 50;
    one JSON line per (system, form), best of two timed calls."""
    import numpy as np
    import torch

    import hyk
    from hyk import workloads as W

    peak = hyk.fp64_peak(0, 300.0)
    n = 65536
    cases = [
        ("oss", W.oss_sys(), W.oss_ics(n, seed=2)[0], None, 2e4, [0, 1, 4, 8, 16, 32]),
        ("cr3bp", W.cr3bp_sys()) + W.cr3bp_ics(n, seed=3) + (50.0, [0, 1, 2, 4, 8, "global"]),
        ("kepler", W.kepler_sys(), W.kepler_ics(4 * n, seed=1), None, 50.0, [0, 1, 2, 4, "global"]),
    ]
    for name, sys_, st, pars, tf, teams in cases:
        s0 = torch.tensor(st, device="cuda")
        for T in teams + ["autotune"]:
            gj = T == "global"  # one thread per trajectory, coefficients in global memory
            at = T == "autotune"  # measured choice (hyk.autotune)
            t_c = time.perf_counter()
            ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=1e-15, team_size=1 if gj else (0 if at else T),
                                           global_jets=gj, autotune=at)
            t_c = time.perf_counter() - t_c
            info = ta.module_info
            ta.propagate_until(tf * 0.01)
            best = 1e30
            for _ in range(2):
                ta.set_time(0.0)
                ta.state[:] = s0
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                ta.propagate_until(tf)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            steps = int(ta.propagate_res_tensors["n_steps"].sum().item())
            fl = info["flops_per_step"] * steps / best
            print(json.dumps({"system": name, "requested_team_size": T, "team_size": info["team_size"],
                              "jets": "global" if info["smem_per_lane"] == 0 else "shared",
                              "block_threads": info["block_lanes"], "ctas_per_sm": info["ctas_per_sm"],
                              "regs": info["regs_per_thread"], "s": best, "trajectory_steps_per_s": steps / best,
                              "fp64_frac_of_measured": fl / peak,
                              **({"autotune_best": ta._autotune["best"], "construct_s": t_c} if at else {})}),
                  flush=True)


def run_plain(args):
    """The plain form (one launch per step, over the unfinished lanes listed
    before each launch) against the persistent kernel, in each system's
    default kernel form: 2^20 Kepler orbits to t = 20, 65536 CR3BP
    trajectories to t = 50 and 65536 outer-solar-system members to end times
    log-uniform in [1e3, 1e5] days; best of two calls, one JSON line per
    (system, mode)."""
    import torch

    import hyk
    from hyk import workloads as W

    cr_st, cr_mu = W.cr3bp_ics(65536, seed=3)
    oss_st, oss_t = W.oss_ics(65536, seed=2)
    cases = [("kepler", W.kepler_sys(), W.kepler_ics(1 << 20, seed=1), None, 20.0),
             ("cr3bp", W.cr3bp_sys(), cr_st, cr_mu, 50.0),
             ("oss", W.oss_sys(), oss_st, None, oss_t)]
    for name, sys_, st, pars, tf in cases:
        for mode in ("persistent", "plain"):
            ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=TOL, prop_mode=mode)
            info = ta.module_info
            best = 1e30
            for _ in range(2):
                ta.set_time(0.0)
                ta.state[:] = st
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                ta.propagate_until(tf)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            steps = int(ta.propagate_res_tensors["n_steps"].sum().item())
            print(json.dumps({"system": name, "mode": mode, "team_size": info["team_size"],
                              "jets": "global" if info["smem_per_lane"] == 0 else "shared", "s": best,
                              "trajectory_steps": steps, "trajectory_steps_per_s": steps / best}), flush=True)


def run_occupancy(args):
    """Lane form with its coefficients in shared memory at every block size
    from 32 to 256 lanes: 2^18 Kepler orbits propagated from t = 0 to 20, at
    tol 1e-9 (order 12) and 1e-15 (order 19); one JSON line per block size
    (resident warps per SM against trajectory-steps/s)."""
    import torch

    import hyk
    from hyk import workloads as W

    n = 1 << 18
    st = W.kepler_ics(n, seed=1)
    for tol in (1e-9, TOL):
        for blk in (32, 64, 96, 128, 160, 192, 224, 256):
            try:
                ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=tol, block_lanes=blk)
            except Exception as e:  # noqa: BLE001 - a block too large for shared memory
                print(json.dumps({"tol": tol, "block_lanes": blk, "skipped": str(e)[:120]}), flush=True)
                continue
            info = ta.module_info
            ta.propagate_until(1.0)
            ta.set_time(0.0)
            ta.state[:] = st
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            ta.propagate_until(20.0)
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            steps = int(ta.propagate_res_tensors["n_steps"].sum().item())
            print(json.dumps({"tol": tol, "order": ta.order, "block_lanes": info["block_lanes"],
                              "ctas_per_sm": info["ctas_per_sm"],
                              "warps_per_sm": info["ctas_per_sm"] * info["block_lanes"] / 32,
                              "smem_per_lane": info["smem_per_lane"], "regs": info["regs_per_thread"],
                              "ms": ms, "trajectory_steps_per_s": steps / ms * 1e3}), flush=True)


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload != "kepler":
        if rank == 0:
            {"serve": run_serve, "pendulum": run_pendulum, "cr3bp-adjoint": run_cr3bp_adjoint, "oss": run_oss,
             "forms": run_forms, "kepler-f32": run_kepler_f32, "occupancy": run_occupancy,
             "plain": run_plain}[args.workload](args)
        return
    import numpy as np
    import torch

    import hyk
    from hyk import workloads as W

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    K, Wm = max(1, args.steps), max(3, args.warmup)
    dt = T_END / K
    n = args.orbits
    st = W.kepler_ics(n, seed=1 + rank)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=TOL, device="cuda:{}".format(dev), team_size=args.team_size)
    info = ta.module_info
    # algorithmic flops per trajectory-step: the measurement contract's count
    # (contract_flops), and the code generator's own, more conservative count
    flops_step = contract_flops(W.kepler_sys(), 19)
    flops_gen = info["flops_per_step"]
    peak = hyk.fp64_peak(dev, 300.0)

    # warm-up on a copy (same kernel, same data)
    wcopy = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=TOL, device="cuda:{}".format(dev), team_size=args.team_size)
    for k in range(Wm):
        wcopy.propagate_until((k + 1) * dt)
    del wcopy
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    # ---- timed: persistent kernel, device-resident ensemble
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    kevs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    steps_per = []
    clk = Clocks(dev)
    barrier()
    t_wall = time.perf_counter()
    for k in range(K):
        evs[k][0].record(stream)
        ta._launch_events = kevs[k]
        ta.propagate_until((k + 1) * dt)
        evs[k][1].record(stream)
        steps_per.append(ta.propagate_res_tensors["n_steps"].sum())
    barrier()
    wall = time.perf_counter() - t_wall
    clocks = clk.stop()
    ta._launch_events = None
    step_ms = [a.elapsed_time(b) for a, b in evs]
    kern_ms = [a.elapsed_time(b) for a, b in kevs]
    n_steps = int(torch.stack(steps_per).sum().item())
    t_gpu = sum(step_ms) / 1e3
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([t_gpu], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_gpu = t.item()
        c = torch.tensor([n_steps], device="cuda", dtype=torch.float64)
        dist.all_reduce(c)
        total_steps = int(c.item())
    else:
        total_steps = n_steps
    value = total_steps / t_gpu
    outcomes_ok = bool((ta.propagate_res_tensors["outcome"] == int(hyk.taylor_outcome.time_limit)).all())
    final_t_ok = bool(np.all(ta.time == T_END))
    alg_flops = flops_step * n_steps
    achieved = alg_flops / (sum(kern_ms) / 1e3)

    # ---- e2e through the public API with host buffers (pinned), same workload
    host_state = torch.tensor(st, dtype=torch.float64).pin_memory()
    out_state = torch.empty_like(host_state).pin_memory()
    out_steps = torch.empty(n, dtype=torch.int64).pin_memory()
    ta2 = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=TOL, device="cuda:{}".format(dev), team_size=args.team_size)
    ta2.propagate_until(dt)  # warm
    ta2.set_time(0.0)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    cur = host_state
    e2e_steps = []
    for k in range(K):
        ta2.state.copy_(cur, non_blocking=True)
        ta2.propagate_until((k + 1) * dt)
        out_state.copy_(ta2.state, non_blocking=True)
        out_steps.copy_(ta2.propagate_res_tensors["n_steps"], non_blocking=True)
        e2e_steps.append(ta2.propagate_res_tensors["n_steps"].sum())
        cur = out_state
    e1.record(stream)
    barrier()
    e2e_t = e0.elapsed_time(e1) / 1e3
    e2e_total = int(torch.stack(e2e_steps).sum().item())
    e2e = {
        "value": e2e_total * world / e2e_t if world > 1 else e2e_total / e2e_t,
        "unit": UNIT,
        "h2d_bytes_per_step": int(host_state.numel() * 8),
        "d2h_bytes_per_step": int(out_state.numel() * 8 + out_steps.numel() * 8),
    }
    del ta2

    # ---- plain (one launch per step) on the same workload, one pass 0..200
    paths = {"persistent": value}
    if not args.no_plain:
        tp = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=TOL, device="cuda:{}".format(dev), prop_mode="plain")
        tp.propagate_until(1.0)
        tp.set_time(0.0)
        tp.state[:] = st
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        tp.propagate_until(T_END)
        b.record(stream)
        barrier()
        ps = int(tp.propagate_res_tensors["n_steps"].sum().item())
        paths["plain"] = ps / (a.elapsed_time(b) / 1e3)
        paths["persistent_over_plain"] = value / paths["plain"]
        # the naive drop-in form: one launch per step over every lane (the
        # reference's batch step called in a loop), finished lanes included
        tp.prop_mode = "plain_inplace"
        tp.set_time(0.0)
        tp.state[:] = st
        barrier()
        a.record(stream)
        tp.propagate_until(T_END)
        b.record(stream)
        barrier()
        ps = int(tp.propagate_res_tensors["n_steps"].sum().item())
        paths["plain_inplace"] = ps / (a.elapsed_time(b) / 1e3)
        paths["persistent_over_plain_inplace"] = value / paths["plain_inplace"]
        del tp

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_sample, 1, T_END)
        parity = parity_checks(dev, K)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": K,
            "warmup": Wm,
            "ms_per_step": t_gpu / K * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded Kepler elements, per-rank seed)",
            "config": {
                "workload": "kepler-2^20 tol=1e-15 t=0..200",
                "orbits_per_gpu": n,
                "order": ta.order,
                "step": "propagate the resident ensemble over {:g} time units (K steps = t 0..200)".format(dt),
                "l2": "inputs larger than L2 (state + bookkeeping ~{:.0f} MB per GPU)".format(n * 21 * 8 / 1e6),
                "block_lanes": info["block_lanes"],
                "regs_per_thread": info["regs_per_thread"],
                "smem_per_lane": info["smem_per_lane"],
                "parallelism": "independent shards of orbits per GPU" if world > 1 else "single GPU",
            },
            "e2e": e2e,
            "paths": paths,
            # per step: bookkeeping init (hyk_prop_init_kernel), the one-step estimate of the
            # longest-first order (hyk_step_kernel), the propagation (hyk_prop_kernel)
            "gpu_launches": 3 * K,
            "roofline": {
                "bound": "fp64",
                "achieved": achieved / 1e12,
                "peak": peak / 1e12,
                "unit": "TFLOP/s",
                "frac": achieved / peak,
                # DRAM bytes per launch: ncu's dram__bytes_read.sum + dram__bytes_write.sum of one
                # 2^17-orbit launch (20.2 MB, one load and one store of each lane's state and
                # bookkeeping; the cold-row buffer stays in L2), scaled by the lanes of this
                # launch (the traffic is per lane)
                "traffic": KEPLER_DRAM_BYTES_PER_LANE * n,
                "traffic_source": "ncu capture of a 2^17-orbit launch, scaled by lanes",
                "kernel": "hyk_prop_kernel (persistent)",
                "flops_per_traj_step": flops_step,
                "flops_per_traj_step_generated": flops_gen,
                "frac_generated": flops_gen * n_steps / (sum(kern_ms) / 1e3) / peak,
                "peak_source": "measured in-process FP64 FMA probe (hyk_fp64_peak), of measured; "
                               "MEASURED_PEAKS.json has no FP64 entry",
            },
            "cpu_baseline": cpu,
            "clocks": clocks,
            "checks": {"all_time_limit": outcomes_ok, "final_time_exact": final_t_ok, "total_traj_steps": total_steps,
                       "parity_1024_orbits": parity},
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
