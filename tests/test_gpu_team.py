"""GPU parity of the team form (several threads per trajectory).

The team form runs the same recurrences, step-size rule and bookkeeping as
the lane form with the work of one trajectory spread over a team of 2..32
threads of a warp; results must equal the oracle's gpu arithmetic bit for
bit, for every team size and both propagation kernels."""

import numpy as np
import pytest
import torch

import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu


def forced():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]


CASES = {
    "pendulum": lambda: (W.pendulum_sys(), W.pendulum_ics(70, seed=31), None, 2.2e-16, 12.0),
    "kepler": lambda: (W.kepler_sys(), W.kepler_ics(70, seed=32), None, 1e-15, 9.0),
    "forced": lambda: (forced(), W.pendulum_ics(40, seed=33), np.full((1, 40), 0.1), 2.2e-16, 6.0),
    "cr3bp": lambda: (W.cr3bp_sys(),) + W.cr3bp_ics(50, seed=34) + (1e-15, 5.0),
}


def res_arrays(ta):
    return {k: v.cpu().numpy() for k, v in ta.propagate_res_tensors.items()}


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("team", [2, 8, 32])
@pytest.mark.parametrize("name", list(CASES))
def test_team_propagate_until_bitwise(oracle, name, team, mode):
    sys_, st, pars, tol, tf = CASES[name]()
    ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=tol, prop_mode=mode, team_size=team)
    assert ta.module_info["team_size"] == team
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st, pars=pars, order=ta.order, mode=1)
    r = o.propagate_until(tf)
    g = res_arrays(ta)
    assert np.array_equal(np.asarray(ta.state), o.state)
    assert np.array_equal(ta.dtime[0], o.t_hi) and np.array_equal(ta.dtime[1], o.t_lo)
    assert np.array_equal(g["n_steps"], r["n_steps"].astype(np.int64))
    assert np.array_equal(g["min_h"], r["min_h"]) and np.array_equal(g["max_h"], r["max_h"])


def test_team_step_grid_for_backward(oracle):
    sys_, st, _, tol, _ = CASES["kepler"]()
    st = st[:, :45]
    ta = hyk.taylor_adaptive_batch(sys_, st, tol=tol, team_size=4)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    for _ in range(2):
        ta.step(write_tc=True)
        oc, h = o.step()
        assert np.array_equal(np.asarray(ta.state), o.state)
        assert np.array_equal(np.array([x[1] for x in ta.step_res]), h)
        assert np.array_equal(ta.tc, o.tc)
    ta.step_backward()
    o.step(backward=True)
    assert np.array_equal(np.asarray(ta.state), o.state)
    ta.propagate_for(3.5, max_delta_t=0.3)
    r = o.propagate_for(3.5, max_delta_t=0.3)
    assert np.array_equal(np.asarray(ta.state), o.state)
    assert np.array_equal(res_arrays(ta)["n_steps"], r["n_steps"].astype(np.int64))
    grid = np.repeat(ta.time.reshape(1, -1), 30, axis=0) + np.linspace(0.0, 6.0, 30).reshape(-1, 1)
    _, out = ta.propagate_grid(grid)
    r = o.propagate_grid(grid)
    assert np.array_equal(out, r["grid"])
    tf = np.where(np.arange(45) % 2 == 0, ta.time + 4.0, ta.time - 4.0)
    ta.propagate_until(tf)
    o.propagate_until(tf)
    assert np.array_equal(np.asarray(ta.state), o.state)


def test_team_c_output_and_max_steps(oracle):
    sys_, st, _, tol, _ = CASES["pendulum"]()
    st = st[:, :33]
    ta = hyk.taylor_adaptive_batch(sys_, st, tol=tol, team_size=16)
    c, _ = ta.propagate_until(5.0, c_output=True)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    o.propagate_until(5.0, c_output=True)
    ts = np.linspace(0.1, 4.9, 7)
    ref = hyk.taylor_adaptive_batch(sys_, st, tol=tol, team_size=1)
    c1, _ = ref.propagate_until(5.0, c_output=True)
    for t in ts:
        assert np.array_equal(c(t), c1(t))
    ta2 = hyk.taylor_adaptive_batch(sys_, st, tol=tol, team_size=16)
    ta2.propagate_until(50.0, max_steps=7)
    assert all(r[3] == 7 for r in ta2.propagate_res)
    o2 = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    o2.propagate_until(50.0, max_steps=7)
    assert np.array_equal(np.asarray(ta2.state), o2.state)


def test_team_sliced_persistent_identical():
    # Time-sliced persistent launches (trajectories stored and resumed) give
    # the same bits as one unbounded launch.
    sys_, st, pars, tol, tf = CASES["cr3bp"]()
    a = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=tol, team_size=8)
    a.propagate_until(tf)
    b = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=tol, team_size=8, prop_mode="plain")
    b.propagate_until(tf)
    assert np.array_equal(np.asarray(a.state), np.asarray(b.state))
    assert torch.equal(a.propagate_res_tensors["n_steps"], b.propagate_res_tensors["n_steps"])


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("team", [4, 16])
def test_team_global_memory_bitwise(oracle, team, mode):
    """Team form with the coefficient regions in global memory (one region per
    team of a fixed resident grid): more trajectories than resident teams, so
    the step and plain kernels loop over lanes; bit-for-bit with the oracle."""
    st = W.kepler_ics(20000, seed=35)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15, prop_mode=mode, team_size=team, global_jets=True)
    info = ta.module_info
    assert info["team_size"] == team and info["smem_per_lane"] == 0
    assert info["n_sm"] * info["ctas_per_sm"] * info["block_lanes"] // team < 20000
    o = oracle.Oracle(W.kepler_sys(), st, order=ta.order, mode=1)
    ta.step(write_tc=True)
    o.step()
    assert np.array_equal(np.asarray(ta.state), o.state) and np.array_equal(ta.tc, o.tc)
    ta.propagate_until(3.0)
    r = o.propagate_until(3.0)
    assert np.array_equal(np.asarray(ta.state), o.state)
    assert np.array_equal(res_arrays(ta)["n_steps"], r["n_steps"].astype(np.int64))


def test_team_global_memory_oss_matches_shared():
    st, t_end = W.oss_ics(400, seed=36)
    grid = np.linspace(0.0, 1.0, 20).reshape(-1, 1) * t_end.reshape(1, -1)
    a = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, team_size=16)
    b = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, team_size=16, global_jets=True)
    _, ga = a.propagate_grid(grid)
    _, gb = b.propagate_grid(grid)
    assert np.array_equal(ga, gb) and torch.equal(a.state, b.state)


@pytest.mark.parametrize("gmem", [False, True])
def test_team_plain_compacted_and_in_place_identical(monkeypatch, gmem):
    """The team form's plain propagation over the compacted list of unfinished
    trajectories, and over all of them in place (a workspace of only the
    counters), gives the persistent form's bits; end times from 1 to 20, so
    that trajectories finish many launches apart."""
    from hyk import _lib

    n = 2000
    st = W.kepler_ics(n, seed=36)
    tf = np.linspace(1.0, 20.0, n)

    def run(mode):
        ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15, prop_mode=mode, team_size=4, global_jets=gmem)
        ta.propagate_until(tf)
        return np.asarray(ta.state), ta.propagate_res

    ref = run("persistent")
    comp = run("plain")
    monkeypatch.setattr(_lib.load(), "hyk_propagate_workspace_size", lambda *a: 256)
    inplace = run("plain")
    for r in (comp, inplace):
        assert np.array_equal(r[0], ref[0]) and r[1] == ref[1]


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("team", [2, 4, 16])
def test_team_cold_rows_bitwise(oracle, team, mode):
    """6-body problem (every state variable read at its current order only):
    the team form with cold state rows (two shared slots per state variable,
    the orders in a global buffer per resident team) against the same form
    without them and against the oracle, bit for bit.  More trajectories
    than resident teams, so the step and plain kernels loop over them."""
    st, _ = W.oss_ics(3000, seed=37)
    a = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, prop_mode=mode, team_size=team)
    ia = a.module_info
    assert ia["team_size"] == team
    assert ia["n_sm"] * ia["ctas_per_sm"] * ia["block_lanes"] // team < 3000
    if team > 2:  # (two threads: 16 trajectories a CTA fit shared memory only with cold rows)
        b = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, prop_mode=mode, team_size=team, cold_rows=False)
        assert ia["smem_per_lane"] < b.module_info["smem_per_lane"]
        assert ia["ctas_per_sm"] > b.module_info["ctas_per_sm"]
    else:
        b = None
    o = oracle.Oracle(W.oss_sys(), st[:, :8], order=a.order, mode=1)
    a.step(write_tc=True)
    o.step()
    assert np.array_equal(np.asarray(a.state)[:, :8], o.state) and np.array_equal(a.tc[..., :8], o.tc)
    if b is not None:
        b.step(write_tc=True)
        assert np.array_equal(a.tc, b.tc) and torch.equal(a.state, b.state)
    grid = np.linspace(0.0, 3000.0, 7).reshape(-1, 1) + a.time.reshape(1, -1)
    _, ga = a.propagate_grid(grid)
    r = o.propagate_grid(grid[:, :8])
    assert np.array_equal(ga[..., :8], r["grid"])
    assert np.array_equal(np.asarray(a.state)[:, :8], o.state)
    if b is not None:
        _, gb = b.propagate_grid(grid)
        assert np.array_equal(ga, gb) and torch.equal(a.state, b.state)
        assert torch.equal(a.propagate_res_tensors["n_steps"], b.propagate_res_tensors["n_steps"])
