"""Continuous-batching server: results identical alone and in a mix, and
identical to a plain batch propagation of the same trajectories."""

import numpy as np
import pytest
import torch

import hyk
from hyk import _lib, serve, workloads as W

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


@pytest.mark.parametrize("mode", ["resident", "slice"])
def test_alone_equals_mix_and_batch(libhyk, mode):
    assert torch.cuda.is_available()
    reqs = make_requests()
    srv = serve.Server(systems(), hbm_budget=64 << 20, slice_iters=16, mode=mode)
    if mode == "resident":
        assert all(isinstance(p, serve.ResidentPool) for p in srv.pools.values())
    mix = {r.rid: r for r in srv.run(reqs, realtime=True)}
    assert len(mix) == len(reqs)
    for r in reqs[:6]:
        alone = serve.Server(systems(), hbm_budget=64 << 20, slice_iters=5, mode=mode).run([r], realtime=False)[0]
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


@pytest.mark.parametrize("mode", ["resident", "slice"])
def test_admission_waits_for_capacity(libhyk, mode):
    # a pool with room for 100 lanes: requests wait until lanes free up
    reqs = [serve.Request("kepler", W.kepler_ics(60, seed=i), 5.0, arrival=0.0, rid=i) for i in range(5)]
    srv = serve.Server({"kepler": (W.kepler_sys(), 1e-15)}, hbm_budget=100 * (6 + 16) * 8, slice_iters=8, mode=mode)
    assert srv.pools["kepler"].C == 100
    res = srv.run(reqs, realtime=False)
    assert sorted(r.rid for r in res) == list(range(5))
    st = serve.latency_stats(res)
    assert st["n"] == 5 and st["p99_ms"] >= st["p50_ms"] > 0


def _pool(**kw):
    return serve.ResidentPool("kepler", W.kepler_sys(), 1e-15, 4096, "cuda:0", **kw)


def _flags(pool):
    return pool.flags.cpu().numpy()


def test_serve_kernel_returns_when_idle(libhyk):
    """The resident kernel's bounded wait: with an empty ring it returns after
    idle_ns on its own, reporting HYK_SERVE_IDLE."""
    pool = _pool(idle_ms=1.0, max_wait_ms=5000.0)
    pool._launch()
    pool.kernel_ev.synchronize()
    assert _flags(pool)[1] & _lib.HYK_SERVE_IDLE
    assert int(pool.words[2].item()) == 0  # nothing in flight


def test_serve_kernel_stop(libhyk):
    """With the stop word set no thread waits: the launch returns at once."""
    pool = _pool(idle_ms=60000.0, max_wait_ms=60000.0)
    pool._launch()
    pool.stop_kernel(wait=True)
    assert _flags(pool)[1] & _lib.HYK_SERVE_STOP


def test_serve_kernel_timeout_while_a_lane_runs(libhyk):
    """A thread that waits max_wait_ns for work returns (HYK_SERVE_TIMEOUT)
    even while another thread still integrates a lane; that lane finishes,
    is counted, and equals a batch propagation of the same trajectory."""
    pool = _pool(idle_ms=60000.0, max_wait_ms=20.0)
    st = W.kepler_ics(1, seed=77)
    req = serve.Request("kepler", st, 500.0, rid=0)
    pool.reserve_requests(1)
    assert pool.admit([req], 0.0) == 1
    pool.kernel_ev.synchronize()
    flags = _flags(pool)
    assert flags[1] & _lib.HYK_SERVE_TIMEOUT
    assert int(pool.done[0].item()) == 1
    res = []
    while not res:
        res = pool.poll(lambda: 0.0, block=True)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    ta.propagate_until(500.0)
    assert np.array_equal(res[0].state, np.asarray(ta.state))
    assert np.array_equal(res[0].n_steps, ta.propagate_res_tensors["n_steps"].cpu().numpy())
