"""Continuous-batching server: results identical alone and in a mix, and
identical to a plain batch propagation of the same trajectories."""

import numpy as np
import pytest
import torch

import hyk
from hyk import serve, workloads as W

pytestmark = pytest.mark.gpu


def systems():
    return {
        "pendulum": (W.pendulum_sys(), 1e-15),
        "kepler": (W.kepler_sys(), 1e-15),
        "cr3bp": (W.cr3bp_sys(), 1e-15),
    }


def make_requests(seed=0, n=24):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        kind = ["pendulum", "kepler", "cr3bp"][i % 3]
        size = int(rng.integers(1, 200))
        tf = float(np.exp(rng.uniform(0.0, np.log(30.0))))
        if kind == "pendulum":
            st, pa = W.pendulum_ics(size, seed=100 + i), None
        elif kind == "kepler":
            st, pa = W.kepler_ics(size, seed=100 + i), None
        else:
            st, pa = W.cr3bp_ics(size, seed=100 + i)
        reqs.append(serve.Request(kind, st, tf, pars=pa, arrival=0.001 * i, rid=i))
    return reqs


def test_alone_equals_mix_and_batch(libhyk):
    assert torch.cuda.is_available()
    reqs = make_requests()
    mix = {r.rid: r for r in serve.Server(systems(), hbm_budget=64 << 20, slice_iters=16).run(reqs, realtime=False)}
    assert len(mix) == len(reqs)
    for r in reqs[:6]:
        alone = serve.Server(systems(), hbm_budget=64 << 20, slice_iters=5).run([r], realtime=False)[0]
        m = mix[r.rid]
        assert np.array_equal(alone.state, m.state) and np.array_equal(alone.n_steps, m.n_steps)
        assert np.array_equal(alone.min_h, m.min_h) and np.array_equal(alone.max_h, m.max_h)
        # and the same as one batch propagation of the request's trajectories
        sys_, tol = systems()[r.system]
        ta = hyk.taylor_adaptive_batch(sys_, r.state, pars=r.pars, tol=tol)
        ta.propagate_until(r.t_final)
        assert np.array_equal(np.asarray(ta.state), m.state)
        assert np.array_equal(ta.propagate_res_tensors["n_steps"].cpu().numpy(), m.n_steps)
        assert np.all(m.outcome == int(hyk.taylor_outcome.time_limit))


def test_admission_waits_for_capacity(libhyk):
    # a pool with room for 100 lanes: requests wait until lanes free up
    reqs = [serve.Request("kepler", W.kepler_ics(60, seed=i), 5.0, arrival=0.0, rid=i) for i in range(5)]
    srv = serve.Server({"kepler": (W.kepler_sys(), 1e-15)}, hbm_budget=100 * (6 + 16) * 8, slice_iters=8)
    assert srv.pools["kepler"].C == 100
    res = srv.run(reqs, realtime=False)
    assert sorted(r.rid for r in res) == list(range(5))
    st = serve.latency_stats(res)
    assert st["n"] == 5 and st["p99_ms"] >= st["p50_ms"] > 0
