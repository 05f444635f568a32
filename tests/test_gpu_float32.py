"""GPU parity of the single-precision integrator (``fp_type=numpy.float32``).

The float kernels and the oracle's float gpu arithmetic perform the same IEEE
binary32 operations in the same order with the same float elementary
functions, so the agreement is bit for bit: states, double-length times,
step counts, min/max step sizes, Taylor coefficients, grid and dense output,
for every kernel form (one thread per trajectory with the coefficients in
shared or in global memory, and the team form).  The reference's own float32
batch tests (heyoka/_test_batch_integrator.py, ``fp_types = [np.float32,
float]``) are mirrored for the behaviour they check.
"""

import numpy as np
import pytest
import torch

import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu
f32 = np.float32


def res_arrays(ta):
    r = ta.propagate_res_tensors
    return {k: v.cpu().numpy() for k, v in r.items()}


def _f32(a):
    return None if a is None else np.asarray(a, dtype=f32)


def _eq(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.array_equal(a, b, equal_nan=True)


CASES = {
    "pendulum": lambda: (W.pendulum_sys(), W.pendulum_ics(256, seed=21), None, 30.0, {}),
    "kepler": lambda: (W.kepler_sys(), W.kepler_ics(256, seed=22), None, 20.0, {}),
    "cr3bp": lambda: (W.cr3bp_sys(),) + W.cr3bp_ics(192, seed=23) + (8.0, {}),
    "cr3bp-team": lambda: (W.cr3bp_sys(),) + W.cr3bp_ics(192, seed=24) + (8.0, {"team_size": 4}),
    "kepler-gmem": lambda: (W.kepler_sys(), W.kepler_ics(256, seed=25), None, 20.0, {"global_jets": True}),
}


def test_float32_module_facts():
    ta = hyk.taylor_adaptive_batch(W.pendulum_sys(), _f32(W.pendulum_ics(8, seed=1)), fp_type=f32)
    assert ta.order == 9 and ta.tol == float(np.finfo(f32).eps)
    assert ta.state.dtype == torch.float32 and ta.fp_type is np.float32
    assert "#define HYK_F32 1" in ta.llvm_state.get_ir()
    assert ta.module_info["smem_per_lane"] % 4 == 0
    assert repr(ta).startswith("C++ datatype            : float")


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("name", list(CASES))
def test_float32_propagate_until_bitwise(oracle, name, mode):
    sys_, st, pars, tf, kw = CASES[name]()
    st, pars = _f32(st), _f32(pars)
    ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, fp_type=f32, prop_mode=mode, **kw)
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st.astype(np.float64), pars=None if pars is None else pars.astype(np.float64),
                      order=ta.order, prec=2, mode=1)
    r = o.propagate_until(tf)
    g = res_arrays(ta)
    assert _eq(np.asarray(ta.state), o.state), name
    assert _eq(ta.dtime[0], o.t_hi) and _eq(ta.dtime[1], o.t_lo)
    assert np.array_equal(g["n_steps"], r["n_steps"].astype(np.int64))
    assert _eq(g["min_h"], r["min_h"]) and _eq(g["max_h"], r["max_h"])
    assert np.all(g["outcome"] == int(hyk.taylor_outcome.time_limit))


def test_float32_step_grid_dense_bitwise(oracle):
    sys_, st, _, _, _ = CASES["kepler"]()
    st = _f32(st[:, :64])
    ta = hyk.taylor_adaptive_batch(sys_, st, fp_type=f32)
    o = oracle.Oracle(sys_, st.astype(np.float64), order=ta.order, prec=2, mode=1)
    for _ in range(3):
        ta.step(write_tc=True)
        oc, h = o.step()
        assert _eq(np.asarray(ta.state), o.state)
        assert _eq(np.array([x[1] for x in ta.step_res]), h)
        assert _eq(ta.tc, o.tc)
    # dense output inside the last step: Horner in float with fused multiply-adds
    d = ta.update_d_output(np.zeros(64, dtype=f32), rel_time=True)
    tc = ta.tc
    lh = np.asarray(ta.last_h, dtype=f32)
    dt = (lh + f32(0)).astype(f32)
    exp = np.empty_like(d)
    for i in range(tc.shape[0]):
        acc = tc[i, -1].astype(np.float64)
        for n in range(tc.shape[1] - 2, -1, -1):
            acc = (acc * dt + tc[i, n]).astype(f32).astype(np.float64)  # product exact in double, one rounding
        exp[i] = acc
    assert np.allclose(d, exp, rtol=0, atol=4 * np.finfo(f32).eps * np.abs(exp).max())
    assert _eq(d, np.asarray(ta.state))  # the step's own end point: the same Horner sum
    ta.step_backward()
    o.step(backward=True)
    assert _eq(np.asarray(ta.state), o.state)
    md = np.linspace(0.01, 0.05, 64).astype(f32)
    ta.step(list(md))
    o.step(md.astype(np.float64))
    assert _eq(np.asarray(ta.state), o.state)
    grid = (np.repeat(ta.time.reshape(1, -1), 40, axis=0) + np.linspace(0.0, 6.0, 40, dtype=f32).reshape(-1, 1))
    grid = grid.astype(f32)
    _, out = ta.propagate_grid(grid)
    r = o.propagate_grid(grid.astype(np.float64))
    assert out.dtype == np.float32
    assert _eq(out, r["grid"])
    assert _eq(np.asarray(ta.state), o.state)


def test_float32_c_output_and_backward(oracle):
    sys_, st, _, _, _ = CASES["pendulum"]()
    st = _f32(st[:, :32])
    tf = np.where(np.arange(32) % 2 == 0, 7.0, -7.0).astype(f32)
    ta = hyk.taylor_adaptive_batch(sys_, st, fp_type=f32)
    c, _ = ta.propagate_until(tf, c_output=True)
    o = oracle.Oracle(sys_, st.astype(np.float64), order=ta.order, prec=2, mode=1)
    r = o.propagate_until(tf.astype(np.float64), c_output=True)
    assert _eq(np.asarray(ta.state), o.state) and np.array_equal(ta.time, tf)
    assert c.tcs.dtype == np.float32
    # the continuous output at every step end reproduces the step's end state
    # (the final time: the propagated state)
    assert np.allclose(c(tf), np.asarray(ta.state), rtol=0, atol=1e-5)


def test_float32_close_to_double():
    """Single precision tracks the double integrator to float accuracy."""
    sys_, st, _, _, _ = CASES["pendulum"]()
    st = _f32(st[:, :128])
    a = hyk.taylor_adaptive_batch(sys_, st, fp_type=f32)
    b = hyk.taylor_adaptive_batch(sys_, st.astype(np.float64))
    a.propagate_until(5.0)
    b.propagate_until(5.0)
    err = np.abs(np.asarray(a.state, dtype=np.float64) - np.asarray(b.state))
    assert err.max() < 2e-4, err.max()
    assert all(r[0] == hyk.taylor_outcome.time_limit for r in a.propagate_res)


def test_float32_reference_propagate_for_semantics():
    """heyoka/_test_batch_integrator.py test_propagate_for, float32 case:
    vector and scalar delta_t / max_delta_t give identical results."""
    ic = np.array([[0.0, 0.1, 0.2, 0.3], [0.25, 0.26, 0.27, 0.28]], dtype=f32)
    x, v = hyk.make_vars("x", "v")
    ta = hyk.taylor_adaptive_batch(sys=[(x, v), (v, -9.8 * hyk.sin(x))], state=ic, fp_type=f32)
    ta.propagate_for([f32(10.0)] * 4)
    st, res = np.asarray(ta.state).copy(), list(ta.propagate_res)
    ta.set_time(f32(0.0))
    ta.state[:] = ic
    ta.propagate_for(f32(10.0))
    assert np.all(np.asarray(ta.state) == st) and ta.propagate_res == res
    ta.set_time(f32(0.0))
    ta.state[:] = ic
    ta.propagate_for([f32(10.0)] * 4, max_delta_t=[f32(1e-4)] * 4)
    st, res = np.asarray(ta.state).copy(), list(ta.propagate_res)
    ta.set_time(f32(0.0))
    ta.state[:] = ic
    ta.propagate_for(f32(10.0), max_delta_t=f32(1e-4))
    assert np.all(np.asarray(ta.state) == st) and ta.propagate_res == res
    assert all(r[3] >= 100000 for r in res)


def test_float32_ensemble_and_copies(oracle):
    from copy import deepcopy
    import pickle

    sys_, st, _, _, _ = CASES["pendulum"]()
    ic = _f32(st[:, :4])
    ta = hyk.taylor_adaptive_batch(sys_, ic, fp_type=f32)

    def gen(t, i):
        t.state[:] = ic + f32(0.01) * i
        return t

    out = hyk.ensemble_propagate_until_batch(ta, 5.0, 6, gen)
    for i, (ti, *_rest) in enumerate(out):
        o = oracle.Oracle(sys_, (ic + f32(0.01) * i).astype(np.float64), order=ta.order, prec=2, mode=1)
        o.propagate_until(5.0)
        assert ti.state.dtype == torch.float32 and _eq(np.asarray(ti.state), o.state)
    ta.propagate_until(1.0)
    for c in (deepcopy(ta), pickle.loads(pickle.dumps(ta))):
        assert c.fp_type is np.float32 and _eq(np.asarray(c.state), np.asarray(ta.state))
        c.propagate_until(2.0)
        ta2 = deepcopy(ta)
        ta2.propagate_until(2.0)
        assert _eq(np.asarray(c.state), np.asarray(ta2.state))


def _pend():
    x, v = hyk.make_vars("x", "v")
    return x, v, [(x, v), (v, -9.8 * hyk.sin(x))]


def _ics(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-1.2, 1.2, n), rng.uniform(-0.5, 0.5, n)]).astype(f32)


def test_float32_reference_events_and_cooldowns():
    """heyoka/_test_batch_integrator.py test_events, float32 case."""
    x, v, sys_ = _pend()

    def cb0(ta, t, d_sgn, bidx):
        pass

    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0.0, 0.001], [0.25, 0.2501]], dtype=f32),
                                   nt_events=[hyk.nt_event_batch(v * v - 1e-6, cb0, fp_type=f32)],
                                   t_events=[hyk.t_event_batch(v, fp_type=f32)], fp_type=f32)
    assert ta.with_events and len(ta.t_events) == 1 and len(ta.nt_events) == 1
    ta.propagate_until([f32(1e9), f32(1e9)])
    assert all(int(r[0]) == -1 for r in ta.propagate_res)
    assert ta.te_cooldowns[0][0] is not None and ta.te_cooldowns[1][0] is not None
    ta.reset_cooldowns(0)
    assert ta.te_cooldowns[0][0] is None and ta.te_cooldowns[1][0] is not None
    ta.reset_cooldowns()
    assert ta.te_cooldowns[0][0] is None and ta.te_cooldowns[1][0] is None


def test_float32_reference_s11n():
    """heyoka/_test_batch_integrator.py test_s11n, float32 case."""
    import pickle

    from test_gpu_events import _Counting, _nt_noop

    x, v, sys_ = _pend()
    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0, 0.01], [0.25, 0.26]], dtype=f32),
                                   nt_events=[hyk.nt_event_batch(v * v - 1e-6, _nt_noop, fp_type=f32)], fp_type=f32)
    for _ in range(4):
        ta.step()
    ta2 = pickle.loads(pickle.dumps(ta))
    assert np.all(ta.state == ta2.state) and np.all(ta.time == ta2.time)
    assert len(ta.t_events) == len(ta2.t_events) and len(ta.nt_events) == len(ta2.nt_events)
    ta.step()
    ta2.step()
    assert np.all(ta.state == ta2.state) and np.all(ta.time == ta2.time)
    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0, 0.01], [0.25, 0.26]], dtype=f32), tol=f32(1e-6), fp_type=f32)
    assert ta.tol == f32(1e-6)
    ta.foo = "hello world"
    ta = pickle.loads(pickle.dumps(ta))
    assert ta.foo == "hello world"

    clb = _Counting()
    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0, 0.01], [0.25, 0.26]], dtype=f32),
                                   t_events=[hyk.t_event_batch(v, callback=clb, fp_type=f32)], fp_type=f32)
    assert id(clb) != id(ta.t_events[0].callback) and ta.t_events[0].callback.n == 0
    ta.propagate_until([f32(100.0), f32(100.0)])
    assert ta.t_events[0].callback.n > 0
    ta2 = pickle.loads(pickle.dumps(ta))
    assert ta.t_events[0].callback.n == ta2.t_events[0].callback.n


def test_float32_nt_events_bitwise_vs_oracle(oracle):
    x, v, sys_ = _pend()
    st = _ics(96, 51)
    recs = []

    def cb_a(ta, t, d_sgn, bidx):
        recs.append((bidx, 0, t, d_sgn))

    def cb_b(ta, t, d_sgn, bidx):
        recs.append((bidx, 1, t, d_sgn))

    ta = hyk.taylor_adaptive_batch(sys_, st, fp_type=f32,
                                   nt_events=[hyk.nt_event_batch(v * v - 1e-4, cb_a, fp_type=f32),
                                              hyk.nt_event_batch(x, cb_b, direction=hyk.event_direction.positive,
                                                                 fp_type=f32)])
    ta.propagate_until(7.5)
    r = oracle.propagate_ev(sys_, [(v * v - 1e-4, False, 0, -1.0), (x, False, 1, -1.0)], st.astype(np.float64), 7.5,
                            order=ta.order, prec=2)
    assert _eq(np.asarray(ta.state), r["state"]) and _eq(ta.time, r["t_hi"])
    assert np.array_equal(ta.propagate_res_tensors["n_steps"].cpu().numpy(), r["n_steps"].astype(np.int64))
    got = sorted(recs)
    want = sorted((int(l), int(i) >> 2, float(t), (int(i) & 3) - 1)
                  for l, i, t in zip(r["rec_lane"], r["rec_info"], r["rec_t_hi"]))
    assert len(got) == len(want) > 96
    assert got == want


def test_float32_terminal_events_bitwise_vs_oracle(oracle):
    x, v, sys_ = _pend()
    st = _ics(80, 52)
    ta = hyk.taylor_adaptive_batch(sys_, st, fp_type=f32,
                                   t_events=[hyk.t_event_batch(v, direction=hyk.event_direction.negative, fp_type=f32)])
    ta.propagate_until(20.0)
    r = oracle.propagate_ev(sys_, [(v, True, -1, -1.0)], st.astype(np.float64), 20.0, order=ta.order, prec=2)
    assert [int(o) for o, *_ in ta.propagate_res] == list(r["outcome"])
    assert _eq(np.asarray(ta.state), r["state"]) and _eq(ta.time, r["t_hi"])
    ta.propagate_until(20.0)
    r2 = oracle.propagate_ev(sys_, [(v, True, -1, -1.0)], r["state"], 20.0, order=ta.order, time=r["t_hi"],
                             time_lo=r["t_lo"], ev_last=r["ev_last"], prec=2)
    assert _eq(ta.time, r2["t_hi"]) and _eq(np.asarray(ta.state), r2["state"])
    assert np.all(ta.time > r["t_hi"])
