"""GPU parity: the CUDA integrator against the CPU oracle (gpu arithmetic).

The kernels and the oracle's "gpu" mode perform the same IEEE operations in
the same order, with the same deterministic elementary functions, so the
expected agreement is bit-for-bit: final states, times, step counts, min/max
step sizes, Taylor coefficients and dense output.  The reference's notebook
pins are checked on the GPU too (step sizes within 2 ulp of the reference's
C-library arithmetic, step counts exact).
"""

import ctypes
import pickle
from copy import copy, deepcopy

import numpy as np
import pytest
import torch

import hyk
from hyk import _lib
from hyk import workloads as W

pytestmark = pytest.mark.gpu


def ulps(a, b):
    return abs(a - b) / np.spacing(max(abs(a), abs(b)))


def pend():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, -9.8 * hyk.sin(x))]


def forced():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]


@pytest.fixture(scope="module", autouse=True)
def _built(libhyk):
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    yield


def res_arrays(ta):
    r = ta.propagate_res_tensors
    return {k: v.cpu().numpy() for k, v in r.items()}


def test_dmath_bitwise_gpu_vs_cpu(libhyk, oracle):
    from hyk import _lib

    rng = np.random.default_rng(7)
    L = oracle.lib()
    cases = [
        (0, rng.uniform(-700, 700, 4096), None),
        (1, np.exp(rng.uniform(-700, 700, 4096)), None),
        (2, rng.uniform(-1e4, 1e4, 4096), None),
        (3, rng.uniform(-1e4, 1e4, 4096), None),
        (4, np.exp(rng.uniform(-20, 20, 4096)), rng.choice([-1.5, -0.5, 2.0, 3.0, -2.0, 0.3, 1.7], 4096)),
        (5, np.exp(rng.uniform(-80, 5, 4096)), np.exp(rng.uniform(-80, 5, 4096))),
        # single precision (float32 integrator)
        (6, rng.uniform(-87, 88, 4096), None),
        (7, np.exp(rng.uniform(-80, 80, 4096)), None),
        (8, rng.uniform(-1e3, 1e3, 4096), None),
        (9, rng.uniform(-1e3, 1e3, 4096), None),
        (10, np.exp(rng.uniform(-10, 10, 4096)), rng.choice([-1.5, -0.5, 2.0, 3.0, -2.0, 0.3, 1.7], 4096)),
        (11, np.exp(rng.uniform(-30, 5, 4096)), np.exp(rng.uniform(-30, 5, 4096))),
        # large arguments: the exact (Payne-Hanek) reduction of sin and cos
        (2, np.ldexp(rng.uniform(-2.0, 2.0, 4096), rng.integers(29, 1024, 4096)), None),
        (3, np.ldexp(rng.uniform(-2.0, 2.0, 4096), rng.integers(29, 1024, 4096)), None),
        (8, np.ldexp(rng.uniform(-2.0, 2.0, 4096), rng.integers(15, 128, 4096)).astype(np.float32).astype(np.float64),
         None),
    ]
    pd = ctypes.POINTER(ctypes.c_double)
    for fn, x, a in cases:
        a = np.zeros_like(x) if a is None else a
        cpu = np.zeros_like(x)
        L.hyko_dm_eval(fn, x.ctypes.data_as(pd), a.ctypes.data_as(pd), cpu.ctypes.data_as(pd), ctypes.c_uint64(len(x)))
        xd, ad = torch.tensor(x, device="cuda"), torch.tensor(a, device="cuda")
        out = torch.empty_like(xd)
        _lib.check(libhyk.hyk_dmath_eval(fn, xd.data_ptr(), ad.data_ptr(), out.data_ptr(), len(x), None))
        torch.cuda.synchronize()
        g = out.cpu().numpy()
        assert np.array_equal(g.view(np.uint64), cpu.view(np.uint64)), fn


def test_notebook_pins_scalar(pins):
    p = pins["pendulum"]
    ta = hyk.taylor_adaptive_batch(pend(), [[0.05], [0.025]])
    assert ta.order == p["order"]
    ta.step()
    oc, h = ta.step_res[0]
    assert oc == hyk.taylor_outcome.success and ulps(h, p["first_h"]) <= 2
    ta.step_backward()
    assert ulps(ta.step_res[0][1], p["back_h"]) <= 2
    ta.set_time(0.0)
    ta.state[:] = [[0.05], [0.025]]
    ta.propagate_for(5.0)
    assert ta.propagate_res[0][3] == p["for5"]["n_steps"] and ta.time[0] == 5.0
    ta.propagate_until(20.0)
    assert ta.propagate_res[0][3] == p["until20"]["n_steps"]
    ta.propagate_until(0.0)
    r = ta.propagate_res[0]
    assert r[0] == hyk.taylor_outcome.time_limit and r[3] == p["until0"]["n_steps"]
    assert ulps(r[1], p["until0"]["min_h"]) < 64 and ulps(r[2], p["until0"]["max_h"]) < 64
    st = np.asarray(ta.state).ravel()
    assert np.allclose(st, p["until0"]["state"], rtol=0, atol=1e-15)


def test_notebook_pins_batch(pins):
    q = pins["forced_pendulum_batch"]
    ta = hyk.taylor_adaptive_batch(forced(), q["state"], pars=q["pars"])
    ta.step()
    assert max(ulps(h, e) for (_, h), e in zip(ta.step_res, q["step_h"])) <= 2
    ta.step([0.010, 0.011, 0.012, 0.013])
    assert all(oc == hyk.taylor_outcome.time_limit for oc, _ in ta.step_res)
    assert np.all(np.round(np.asarray(ta.state), 8) == q["after_clamped_step"]["state_8digits"])
    ta.propagate_for([10.0, 11.0, 12.0, 13.0])
    assert [r[3] for r in ta.propagate_res] == [e["n_steps"] for e in q["for"]["res"]]
    ta.propagate_until([20.0, 21.0, 22.0, 23.0])
    assert [r[3] for r in ta.propagate_res] == [e["n_steps"] for e in q["until"]["res"]]
    assert np.all(np.round(np.asarray(ta.state), 8) == q["until"]["state_8digits"])
    ta.set_time([0.0] * 4)
    ta.state[:] = q["state"]
    g = np.repeat(np.linspace(0, 100, 1000), 4).reshape(1000, -1)
    _, out = ta.propagate_grid(g)
    assert [r[3] for r in ta.propagate_res] == [e["n_steps"] for e in q["grid"]["res"]]
    assert out.shape == (1000, 2, 4) and np.all(np.isfinite(out))
    ta.set_time([0.0] * 4)
    ta.state[:] = q["state"]
    ta.step(write_tc=True)
    assert np.all(ta.tc[:, 0, :] == np.array(q["tc_order0"]))
    d = ta.update_d_output([0.01, 0.02, 0.03, 0.04])
    assert np.all(np.round(d, 8) == q["d_output_8digits"])
    ta.set_time([0.0] * 4)
    ta.state[:] = q["state"]
    c_out, _ = ta.propagate_until(q["c_output"]["t"], c_output=True)
    assert np.all(np.round(c_out([0.01, 0.02, 0.03, 0.04]), 8) == q["c_output"]["at_0.01..0.04_8digits"])
    c_arr = c_out([[0.01, 0.02, 0.03, 0.04], [1.01, 1.02, 1.03, 1.04], [2.01, 2.02, 2.03, 2.04]])
    assert c_arr.shape == (3, 2, 4)
    assert abs(c_arr[0, 1, 2] - q["c_output"]["c_arr_0_1_2"]) <= 1e-14


CASES = {
    "pendulum": lambda: (W.pendulum_sys(), W.pendulum_ics(200, seed=11), None, 2.2e-16, 30.0),
    "kepler": lambda: (W.kepler_sys(), W.kepler_ics(200, seed=12), None, 1e-15, 20.0),
    "forced": lambda: (forced(), W.pendulum_ics(96, seed=13), np.full((1, 96), 0.1), 2.2e-16, 15.0),
    "cr3bp": lambda: (W.cr3bp_sys(),) + W.cr3bp_ics(160, seed=14) + (1e-15, 8.0),
}


@pytest.mark.parametrize("mode", ["persistent", "plain", "plain_inplace"])
@pytest.mark.parametrize("name", list(CASES))
def test_propagate_until_bitwise(oracle, name, mode):
    sys_, st, pars, tol, tf = CASES[name]()
    ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=tol, prop_mode=mode)
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st, pars=pars, order=ta.order, mode=1)
    r = o.propagate_until(tf)
    g = res_arrays(ta)
    assert np.array_equal(np.asarray(ta.state), o.state), name
    assert np.array_equal(ta.dtime[0], o.t_hi) and np.array_equal(ta.dtime[1], o.t_lo)
    assert np.array_equal(g["n_steps"], r["n_steps"].astype(np.int64))
    assert np.array_equal(g["min_h"], r["min_h"]) and np.array_equal(g["max_h"], r["max_h"])
    assert np.all(g["outcome"] == int(hyk.taylor_outcome.time_limit))


def test_propagate_for_grid_and_step_bitwise(oracle):
    sys_, st, pars, tol, _ = CASES["kepler"]()
    st = st[:, :64]
    ta = hyk.taylor_adaptive_batch(sys_, st, tol=tol)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    for _ in range(3):
        ta.step(write_tc=True)
        oc, h = o.step()
        assert np.array_equal(np.asarray(ta.state), o.state)
        assert np.array_equal(np.array([x[1] for x in ta.step_res]), h)
        assert np.array_equal(ta.tc, o.tc)
    ta.step_backward()
    o.step(backward=True)
    assert np.array_equal(np.asarray(ta.state), o.state)
    md = np.linspace(0.01, 0.05, 64)
    ta.step(list(md))
    o.step(md)
    assert np.array_equal(np.asarray(ta.state), o.state)
    ta.propagate_for(3.5, max_delta_t=0.3)
    r = o.propagate_for(3.5, max_delta_t=0.3)
    assert np.array_equal(np.asarray(ta.state), o.state)
    assert np.array_equal(res_arrays(ta)["n_steps"], r["n_steps"].astype(np.int64))
    grid = np.repeat(ta.time.reshape(1, -1), 40, axis=0) + np.linspace(0.0, 6.0, 40).reshape(-1, 1)
    _, out = ta.propagate_grid(grid)
    r = o.propagate_grid(grid)
    assert np.array_equal(out, r["grid"])
    assert np.array_equal(np.asarray(ta.state), o.state)


def test_backward_and_mixed_directions(oracle):
    sys_, st, _, tol, _ = CASES["pendulum"]()
    st = st[:, :32]
    tf = np.where(np.arange(32) % 2 == 0, 7.0, -7.0)
    ta = hyk.taylor_adaptive_batch(sys_, st, tol=tol)
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    o.propagate_until(tf)
    assert np.array_equal(np.asarray(ta.state), o.state)
    assert np.array_equal(ta.time, tf)


def test_scalar_and_vector_arguments_identical():
    sys_, st, _, tol, _ = CASES["pendulum"]()
    st = st[:, :16]
    a = hyk.taylor_adaptive_batch(sys_, st, tol=tol)
    b = hyk.taylor_adaptive_batch(sys_, st, tol=tol)
    a.propagate_for([10.0] * 16, max_delta_t=[0.05] * 16)
    b.propagate_for(10.0, max_delta_t=0.05)
    assert np.array_equal(np.asarray(a.state), np.asarray(b.state))
    assert a.propagate_res == b.propagate_res


def test_plain_and_persistent_identical():
    sys_, st, _, tol, tf = CASES["kepler"]()
    a = hyk.taylor_adaptive_batch(sys_, st, tol=tol, prop_mode="plain")
    b = hyk.taylor_adaptive_batch(sys_, st, tol=tol, prop_mode="persistent")
    a.propagate_until(tf)
    b.propagate_until(tf)
    assert np.array_equal(np.asarray(a.state), np.asarray(b.state))
    assert a.propagate_res == b.propagate_res


def test_max_steps_step_limit(oracle):
    sys_, st, _, tol, _ = CASES["pendulum"]()
    st = st[:, :8]
    ta = hyk.taylor_adaptive_batch(sys_, st, tol=tol)
    ta.propagate_until(50.0, max_steps=5)
    assert all(r[0] == hyk.taylor_outcome.step_limit and r[3] == 5 for r in ta.propagate_res)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    o.propagate_until(50.0, max_steps=5)
    assert np.array_equal(np.asarray(ta.state), o.state)


def test_zero_duration_and_errors():
    sys_, st, _, tol, _ = CASES["pendulum"]()
    ta = hyk.taylor_adaptive_batch(sys_, st[:, :4], tol=tol)
    ta.propagate_until(0.0)
    assert all(r == (hyk.taylor_outcome.time_limit, np.inf, 0.0, 0) for r in ta.propagate_res)
    with pytest.raises(ValueError, match="non-finite"):
        ta.propagate_until(np.inf)
    with pytest.raises(ValueError, match="max_delta_t"):
        ta.propagate_until(1.0, max_delta_t=-1.0)
    with pytest.raises(TypeError, match="cannot be used as a step callback"):
        ta.propagate_until(1.0, callback="hello world")
    with pytest.raises(ValueError, match="dimension of 1"):
        ta.propagate_grid(np.array([], dtype=float))
    with pytest.raises(ValueError, match="number of columns is 2"):
        ta.propagate_grid(np.array([[1.0, 2.0], [3.0, 4.0]]))
    with pytest.raises(ValueError, match="first element"):
        ta.propagate_grid(np.ones((3, 4)))
    with pytest.raises(ValueError, match="expected number of dimensions is 2"):
        hyk.taylor_adaptive_batch(sys_, [0.1, 0.2])
    with pytest.raises(ValueError, match="expected array shape is \\(n, 4\\)"):
        hyk.taylor_adaptive_batch(forced(), st[:, :4], pars=[[0.1, 0.2]])
    with pytest.raises(ValueError, match="expected array shape is \\(4\\)"):
        hyk.taylor_adaptive_batch(sys_, st[:, :4], time=[0.0])


def test_non_finite_state_stops_lane(oracle):
    """With batch_semantics="lane" a non-finite state stops only its lane (the
    default, the reference's whole-batch stop, is tested in
    test_gpu_batch_semantics.py)."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, hyk.log(x))]
    ta = hyk.taylor_adaptive_batch(sys_, [[-1.0, 1.0], [0.0, 0.0]], batch_semantics="lane")
    ta.propagate_until(0.5)
    res = ta.propagate_res
    assert res[0][0] == hyk.taylor_outcome.err_nf_state
    assert res[1][0] == hyk.taylor_outcome.time_limit


def test_dtime_and_copies():
    sys_, st, _, tol, _ = CASES["pendulum"]()
    ta = hyk.taylor_adaptive_batch(sys_, st[:, :2], tol=tol)
    assert np.all(ta.dtime[0] == 0) and np.all(ta.dtime[1] == 0)
    with pytest.raises(ValueError):
        ta.dtime[0][0] = 0.5
    ta.step()
    ta.propagate_for(1000.1)
    assert not np.all(ta.dtime[1] == 0)
    ta.set_dtime(1.0, 0.5)
    assert np.all(ta.dtime[0] == 1.5) and np.all(ta.dtime[1] == 0)
    ta.set_dtime([1.0, 2.0], [0.5, 0.25])
    assert np.all(ta.dtime[0] == [1.5, 2.25])
    with pytest.raises(TypeError, match="same type"):
        ta.set_dtime([1.0, 2.0], 0.5)
    ta.bar = [1]
    assert copy(ta).bar is ta.bar and deepcopy(ta).bar is not ta.bar
    dc = deepcopy(ta)
    dc.state[0, 0] += 1
    assert dc.state[0, 0].item() != ta.state[0, 0].item()
    pk = pickle.loads(pickle.dumps(ta))
    pk.step()
    ta.step()
    assert np.array_equal(np.asarray(pk.state), np.asarray(ta.state))


def test_d_output_at_current_time():
    sys_, st, _, tol, _ = CASES["pendulum"]()
    ta = hyk.taylor_adaptive_batch(sys_, st[:, :4], tol=tol)
    ta.step(write_tc=True)
    ta.update_d_output(ta.time)
    assert np.allclose(ta.d_output, np.asarray(ta.state), rtol=1e-15 * 10, atol=1e-15 * 10)
    ta.update_d_output(0.0, rel_time=True)
    assert np.allclose(ta.d_output, np.asarray(ta.state), rtol=1e-15 * 10, atol=1e-15 * 10)


def test_c_output_matches_oracle(oracle):
    sys_, st, pars = forced(), W.pendulum_ics(8, seed=3), np.full((1, 8), 0.12)
    tf = np.linspace(5.0, 9.0, 8)
    ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars)
    c_out, _ = ta.propagate_until(tf, c_output=True)
    o = oracle.Oracle(sys_, st, pars=pars, order=ta.order, mode=1)
    r = o.propagate_until(tf, c_output=True)
    assert c_out.n_steps == r["n_iter"]
    assert np.array_equal(c_out.tcs, r["c_tcs"]) and np.array_equal(c_out.times, r["c_thi"])
    vals = c_out(np.linspace(0.0, 4.9, 8))
    assert np.all(np.isfinite(vals))
    # at the final time of each lane the continuous output is the final state
    assert np.allclose(c_out(tf), np.asarray(ta.state), rtol=1e-14, atol=1e-15)


def test_pin_arithmetic_module_close_to_oracle_pin(oracle):
    sys_, st, _, tol, tf = CASES["kepler"]()
    ta = hyk.taylor_adaptive_batch(sys_, st, tol=tol, pin_arith=True)
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=0)
    r = o.propagate_until(tf)
    rel = np.max(np.abs(np.asarray(ta.state) - o.state), axis=0) / np.max(np.abs(o.state), axis=0)
    assert rel.max() <= 1e-12
    assert np.mean(res_arrays(ta)["n_steps"] == r["n_steps"]) >= 0.99


@pytest.mark.parametrize("what", ["until", "grid", "c_output"])
def test_plain_compacted_in_place_and_persistent_identical(monkeypatch, what):
    """The plain form steps a compacted list of the unfinished lanes when its
    workspace holds the list, and every lane in place when it holds only the
    counters; both give the persistent form's bits (lanes with end times from
    1 to 20, so that they finish many launches apart)."""
    sys_ = W.kepler_sys()
    n = 3000
    st = W.kepler_ics(n, seed=5)
    tf = np.linspace(1.0, 20.0, n)
    grid = np.linspace(0.0, 1.0, 7).reshape(-1, 1) * tf.reshape(1, -1)

    def run(mode):
        ta = hyk.taylor_adaptive_batch(sys_, st, tol=1e-15, prop_mode=mode)
        if what == "grid":
            out = ta.propagate_grid(grid)[1]
        elif what == "c_output":
            c = ta.propagate_until(tf, c_output=True)[0]
            out = c(0.5 * tf)
        else:
            ta.propagate_until(tf)
            out = None
        return np.asarray(ta.state), ta.propagate_res, out

    ref = run("persistent")
    comp = run("plain")
    L = _lib.load()
    monkeypatch.setattr(L, "hyk_propagate_workspace_size", lambda *a: 256)
    inplace = run("plain")
    for r in (comp, inplace):
        assert np.array_equal(r[0], ref[0])
        assert r[1] == ref[1]
        if ref[2] is not None:
            assert np.array_equal(r[2], ref[2], equal_nan=True)
