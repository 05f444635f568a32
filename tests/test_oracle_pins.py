"""The CPU oracle against the reference's own known-answer outputs.

The reference cannot run here; its notebooks' recorded outputs
(tests/golden/notebook_pins.json, extracted by tests/golden/make_golden.py)
pin the oracle: step sizes bit-exact, step counts exact, min/max step sizes
to a few ulp (they sit at the end of long chaotic or near-chaotic runs, where
the reference's exact operation order, which is not observable, moves the
last bits), printed 8-digit states exactly.
"""

import os

import numpy as np
import pytest

import hyk
from hyk.decompose import order_from_tol


def traj_rel_err(a, b):
    """Per-trajectory relative error: max |a - b| over the state / max |b|."""
    return np.max(np.abs(a - b), axis=0) / np.max(np.abs(b), axis=0)


def ulps(a, b):
    return abs(a - b) / np.spacing(max(abs(a), abs(b)))


def pend():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, -9.8 * hyk.sin(x))]


def forced():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]


def test_order_rule(pins):
    assert order_from_tol(2.220446049250313e-16) == pins["pendulum"]["order"] == 20
    assert order_from_tol(1e-9) == pins["pendulum_tol1e-9"]["order"] == 12
    assert order_from_tol(1e-15) == 19
    with pytest.raises(ValueError):
        order_from_tol(-1.0)


@pytest.mark.parametrize("mode", [0, 1])
def test_scalar_pendulum_steps(oracle, pins, mode):
    p = pins["pendulum"]
    o = oracle.Oracle(pend(), [[0.05], [0.025]], order=20, mode=mode)
    # pin arithmetic reproduces the reference's step sizes bit for bit; the
    # gpu arithmetic's own exp/log differ from the C library by at most 2 ulp
    tol_ulp = 0 if mode == 0 else 2
    oc, h = o.step()
    assert ulps(h[0], p["first_h"]) <= tol_ulp and oc[0] == hyk.taylor_outcome.success
    oc, h = o.step(backward=True)
    assert ulps(h[0], p["back_h"]) <= tol_ulp
    oc, h = o.step(0.01)
    assert h[0] == 0.01 and oc[0] == hyk.taylor_outcome.time_limit
    oc, h = o.step(-0.02)
    assert h[0] == -0.02 and oc[0] == hyk.taylor_outcome.time_limit
    assert ulps(o.t_hi[0], p["after_clamped_steps"]["time"]) <= 16 * tol_ulp
    assert np.all(np.round(o.state.ravel(), 8) == p["after_clamped_steps"]["state_8digits"])


def test_scalar_pendulum_propagate(oracle, pins):
    p = pins["pendulum"]
    o = oracle.Oracle(pend(), [[0.05], [0.025]], order=20, mode=0)
    r = o.propagate_for(5.0)
    assert r["n_steps"][0] == p["for5"]["n_steps"]
    assert r["min_h"][0] == p["for5"]["min_h"] and r["max_h"][0] == p["for5"]["max_h"]
    assert r["outcome"][0] == hyk.taylor_outcome.time_limit and o.t_hi[0] == 5.0
    r = o.propagate_until(20.0)
    assert r["n_steps"][0] == p["until20"]["n_steps"]
    assert r["min_h"][0] == p["until20"]["min_h"]
    assert ulps(r["max_h"][0], p["until20"]["max_h"]) <= 4
    r = o.propagate_until(0.0)
    assert r["n_steps"][0] == p["until0"]["n_steps"]
    assert ulps(r["min_h"][0], p["until0"]["min_h"]) <= 4
    assert ulps(r["max_h"][0], p["until0"]["max_h"]) <= 4
    # forward 20 and back: the state returns to the initial condition within a few ulp
    assert np.allclose(o.state.ravel(), p["until0"]["state"], rtol=0, atol=1e-16 * 8)


def test_scalar_pendulum_grid(oracle, pins):
    p = pins["pendulum"]["grid"]
    o = oracle.Oracle(pend(), [[0.05], [0.025]], order=20, mode=0)
    r = o.propagate_grid(np.array(p["grid"]).reshape(-1, 1))
    assert r["n_steps"][0] == p["n_steps"]
    assert r["max_h"][0] == p["max_h"]
    assert ulps(r["min_h"][0], p["min_h"]) <= 4
    out = r["grid"][:, :, 0]
    assert np.all(np.round(out, 8) == np.array(p["out_8digits"]))
    assert np.all(out[0] == [0.05, 0.025])


def test_tol_1e9_round_trip(oracle, pins):
    p = pins["pendulum_tol1e-9"]
    o = oracle.Oracle(pend(), [[0.05], [0.025]], order=order_from_tol(p["tol"]), mode=0)
    o.propagate_until(10.0)
    o.propagate_until(0.0)
    # At tol 1e-9 the round-trip error (~1e-12) is truncation error, which
    # the algorithm determines: the reference's printed state is reproduced
    # to a relative 1e-12 of the error itself.
    err = o.state.ravel() - np.array([0.05, 0.025])
    ref = np.array(p["state_after_10_and_back"]) - np.array([0.05, 0.025])
    assert np.all(np.abs(err - ref) <= 1e-3 * np.abs(ref))


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_forced_pendulum(oracle, pins, mode):
    q = pins["forced_pendulum_batch"]
    o = oracle.Oracle(forced(), q["state"], pars=q["pars"], order=20, mode=mode)
    oc, h = o.step()
    assert max(ulps(a, b) for a, b in zip(h, q["step_h"])) <= (0 if mode == 0 else 2)
    o.step([0.010, 0.011, 0.012, 0.013])
    assert np.all(np.round(o.state, 8) == q["after_clamped_step"]["state_8digits"])
    assert np.all(np.round(o.t_hi, 8) == q["after_clamped_step"]["time_8digits"])
    r = o.propagate_for([10.0, 11.0, 12.0, 13.0])
    for i, e in enumerate(q["for"]["res"]):
        assert r["n_steps"][i] == e["n_steps"]
        assert abs(r["min_h"][i] - e["min_h"]) <= 1e-14 * e["min_h"]
        assert abs(r["max_h"][i] - e["max_h"]) <= 1e-14 * e["max_h"]
    assert np.all(np.round(o.state, 8) == q["for"]["state_8digits"])
    r = o.propagate_until([20.0, 21.0, 22.0, 23.0])
    for i, e in enumerate(q["until"]["res"]):
        assert r["n_steps"][i] == e["n_steps"]
        assert abs(r["min_h"][i] - e["min_h"]) <= 1e-13 * e["min_h"]
        assert abs(r["max_h"][i] - e["max_h"]) <= 1e-13 * e["max_h"]
    assert np.all(np.round(o.state, 8) == q["until"]["state_8digits"])
    assert np.all(o.t_hi == [20.0, 21.0, 22.0, 23.0])


def test_batch_forced_pendulum_grid(oracle, pins):
    q = pins["forced_pendulum_batch"]
    o = oracle.Oracle(forced(), q["state"], pars=q["pars"], order=20, mode=0)
    g = np.repeat(np.linspace(0, 100, 1000), 4).reshape(1000, -1)
    r = o.propagate_grid(g)
    for i, e in enumerate(q["grid"]["res"]):
        assert r["n_steps"][i] == e["n_steps"]
        # t = 100 of a chaotic system: agreement to 1e-12 relative
        assert abs(r["min_h"][i] - e["min_h"]) <= 1e-12 * e["min_h"]
        assert abs(r["max_h"][i] - e["max_h"]) <= 1e-12 * e["max_h"]
    assert np.all(np.isfinite(r["grid"]))


def test_batch_dense_and_continuous_output(oracle, pins):
    q = pins["forced_pendulum_batch"]
    o = oracle.Oracle(forced(), q["state"], pars=q["pars"], order=20, mode=0)
    o.step()
    assert np.all(o.tc[:, 0, :] == np.array(q["tc_order0"]))
    # update_d_output(t) for absolute t right after one step from t = 0:
    # Horner at offset t (the step started at 0).
    dt = np.array([0.01, 0.02, 0.03, 0.04])
    tc = o.tc
    out = np.zeros((2, 4))
    for i in range(2):
        acc = tc[i, -1]
        for n in range(tc.shape[1] - 2, -1, -1):
            acc = acc * dt + tc[i, n]
        out[i] = acc
    assert np.all(np.round(out, 8) == q["d_output_8digits"])
    # continuous output over [0, 10.x]: value at t = 0.03 of lane 2
    o = oracle.Oracle(forced(), q["state"], pars=q["pars"], order=20, mode=0)
    r = o.propagate_until(q["c_output"]["t"], c_output=True)
    tcs, thi = r["c_tcs"], r["c_thi"]
    lane, t = 2, 0.03
    k = np.searchsorted(thi[:-1, lane], t, side="right") - 1
    d = t - thi[k, lane]
    acc = tcs[k, 1, -1, lane]
    for n in range(tcs.shape[2] - 2, -1, -1):
        acc = acc * d + tcs[k, 1, n, lane]
    assert abs(acc - q["c_output"]["c_arr_0_1_2"]) <= 2 * np.spacing(acc)


def test_gpu_arith_mode_matches_pin_mode(oracle):
    """The GPU arithmetic (FMA, reciprocals) changes only the last bits."""
    from hyk import workloads as W

    st = W.kepler_ics(32)
    a = oracle.Oracle(W.kepler_sys(), st, order=19, mode=0)
    b = oracle.Oracle(W.kepler_sys(), st, order=19, mode=1)
    ra, rb = a.propagate_until(20.0), b.propagate_until(20.0)
    assert np.max(traj_rel_err(b.state, a.state)) < 1e-12
    assert np.all(ra["n_steps"] == rb["n_steps"])


def test_vector_and_scalar_overloads_identical(oracle):
    o1 = oracle.Oracle(pend(), [[0.0, 0.1, 0.2, 0.3], [0.25, 0.26, 0.27, 0.28]], order=20)
    o2 = oracle.Oracle(pend(), [[0.0, 0.1, 0.2, 0.3], [0.25, 0.26, 0.27, 0.28]], order=20)
    r1 = o1.propagate_for([10.0] * 4, max_delta_t=[1e-1] * 4)
    r2 = o2.propagate_for(10.0, max_delta_t=1e-1)
    assert np.all(o1.state == o2.state)
    for k in ("n_steps", "min_h", "max_h", "outcome"):
        assert np.all(r1[k] == r2[k])


def test_ensemble_equals_serial(oracle):
    from hyk import workloads as W

    st = W.pendulum_ics(24, seed=5)
    ens = oracle.ensemble_until(W.pendulum_sys(), st, None, 0.0, 20.0, order=20, batch=4, n_threads=4, mode=0)
    for b in range(6):
        o = oracle.Oracle(W.pendulum_sys(), st[:, 4 * b: 4 * b + 4], order=20, mode=0)
        r = o.propagate_until(20.0)
        assert np.all(o.state == ens["state"][:, 4 * b: 4 * b + 4])
        assert np.all(r["n_steps"] == ens["n_steps"][4 * b: 4 * b + 4])


def test_max_steps_and_zero_duration(oracle):
    o = oracle.Oracle(pend(), [[0.05, 0.06], [0.025, 0.02]], order=20)
    r = o.propagate_until(10.0, max_steps=3)
    assert np.all(r["outcome"] == hyk.taylor_outcome.step_limit)
    assert np.all(r["n_steps"] == 3)
    o.t_lo[:] = 0.0  # a time with no low part: the target is exactly the current time
    r = o.propagate_until(o.t_hi.copy())
    assert np.all(r["outcome"] == hyk.taylor_outcome.time_limit)
    assert np.all(r["n_steps"] == 0) and np.all(r["min_h"] == np.inf) and np.all(r["max_h"] == 0)


def test_non_finite_state(oracle):
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, hyk.log(x))]  # log of a negative number -> NaN
    o = oracle.Oracle(sys_, [[-1.0, 1.0], [0.0, 0.0]], order=20)
    r = o.propagate_until(1.0)
    assert r["outcome"][0] == hyk.taylor_outcome.err_nf_state


def test_quad_reference_error_kepler(oracle):
    """Error of the double-precision runs against a binary128 run at tol 1e-32."""
    from hyk import workloads as W

    st = W.kepler_ics(8)
    d = oracle.Oracle(W.kepler_sys(), st, order=19, mode=1)
    q = oracle.Oracle(W.kepler_sys(), st, order=order_from_tol(1e-32), prec=1, mode=0)
    d.propagate_until(10.0)
    q.propagate_until(10.0)
    assert np.max(traj_rel_err(d.state, q.state)) < 1e-12


def test_binary128_fixture_kepler_benchmark_orbits(oracle):
    """The binary128 states of 1024 benchmark orbits (tests/golden/
    kepler_t200_quad_1024.npz, made by make_kepler_quad.py): a re-run of the
    first 16 at tol 1e-28 (order 33) agrees with them to 1e-15 at t = 50 and
    t = 200, and
    on the first 256 orbits the gpu and the reference (pin) arithmetic are
    equally far from them at t = 200 (the fixture's use in the GPU tests):
    the same median and 90th percentile within 25 %.  The maximum of 256
    draws of this heavy-tailed error is a lottery (a few orbits amplify
    rounding most, and which of them the rounding of one arithmetic hits
    hardest is not the same for the other): it is compared within 3x."""
    from hyk import workloads as W

    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kepler_t200_quad_1024.npz"))
    st = np.ascontiguousarray(W.kepler_ics(1 << 20, seed=1)[:, fx["idx"]])
    q = oracle.Oracle(W.kepler_sys(), st[:, :16], order=order_from_tol(1e-28), prec=1, mode=0)
    for t in (50.0, 200.0):
        q.propagate_until(t)
        assert np.max(traj_rel_err(q.state, fx["state_t{:g}".format(t)][:, :16])) <= 1e-15
    err = {}
    for mode in (0, 1):
        o = oracle.Oracle(W.kepler_sys(), st[:, :256], order=19, mode=mode)
        o.propagate_until(200.0)
        err[mode] = traj_rel_err(o.state, fx["state_t200"][:, :256])
    assert np.median(err[1]) <= 1.25 * np.median(err[0])
    assert np.quantile(err[1], 0.9) <= 1.25 * np.quantile(err[0], 0.9)
    assert err[1].max() <= 3.0 * err[0].max()
    assert err[0].max() > 1e-12  # the reference arithmetic's own error at this horizon


def test_high_accuracy_oracle_close_to_quad(oracle):
    """The oracle's high-accuracy mode (compensated summation in the state
    update) stays within 1e-12 of the binary128 restatement over 20 time
    units of Kepler orbits, like the default mode."""
    from hyk import workloads as W

    st = W.kepler_ics(8, seed=52)
    q = oracle.Oracle(W.kepler_sys(), st, order=38, prec=1, mode=0)
    q.propagate_until(20.0)
    for mode in (1, 3):
        o = oracle.Oracle(W.kepler_sys(), st, order=19, mode=mode)
        o.propagate_until(20.0)
        assert np.max(np.abs(o.state - q.state)) < 1e-12


def test_single_precision_functions_accuracy(oracle):
    """The float versions of the deterministic functions (float32
    integrator): within 2 ulp of float (pow 3, the step-size rho 4) against float64 numpy
    on their ranges of use."""
    import ctypes

    L = oracle.lib()
    pd = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(0)

    def ev(fn, x, a=None):
        x = np.ascontiguousarray(x, dtype=np.float32).astype(np.float64)
        a = np.zeros_like(x) if a is None else np.ascontiguousarray(a, dtype=np.float32).astype(np.float64)
        out = np.zeros_like(x)
        L.hyko_dm_eval(fn, x.ctypes.data_as(pd), a.ctypes.data_as(pd), out.ctypes.data_as(pd), ctypes.c_uint64(len(x)))
        return x, a, out

    def ulps(got, ref):
        sp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
        return np.max(np.abs(got - ref) / sp)

    x, _, o = ev(6, rng.uniform(-87, 88, 20000))
    assert ulps(o, np.exp(x)) <= 2
    x, _, o = ev(7, np.exp(rng.uniform(-80, 80, 20000)))
    assert ulps(o, np.log(x)) <= 2
    x, _, o = ev(8, rng.uniform(-1e3, 1e3, 20000))
    assert ulps(o, np.sin(x)) <= 2
    x, _, o = ev(9, x)
    assert ulps(o, np.cos(x)) <= 2
    x, a, o = ev(10, np.exp(rng.uniform(-10, 10, 20000)), rng.choice([-1.5, -0.5, 2.0, 3.0, 0.3, 1.7], 20000))
    assert ulps(o, x**a) <= 3
    m, q, o = ev(11, np.exp(rng.uniform(-30, 5, 2000)), np.exp(rng.uniform(-30, 5, 2000)))
    assert ulps(o, np.minimum((1 / m) ** (1 / 9), (1 / q) ** (1 / 8))) <= 4  # the step-size factor


def test_sincos_large_arguments_exact_reduction(oracle):
    """sin and cos beyond |x| = 2^30 (the reduction of Payne and Hanek in
    hyk_dmath.h): within 2 ulp of 2000-bit references over the whole double
    range, including arguments next to multiples of pi/2 (the double closest
    to one, 6381956970095103 2^797, among them), in double and in single
    precision."""
    import ctypes

    mpmath = pytest.importorskip("mpmath")
    L = oracle.lib()
    pd = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(11)
    xs = list(np.ldexp(rng.uniform(1.0, 2.0, 600), rng.integers(30, 1024, 600)))
    xs += [2.0**30, -(2.0**30), np.nextafter(2.0**30, 0.0), 1e22, 1e300, -1.7e308, np.ldexp(6381956970095103.0, 797)]
    mpmath.mp.prec = 2000
    for e in rng.integers(30, 1000, 100):  # doubles next to k pi/2
        k = mpmath.floor(mpmath.ldexp(mpmath.mpf(rng.uniform(1.0, 2.0)), int(e)) / (mpmath.pi / 2))
        xs.append(float(k * mpmath.pi / 2))
    x = np.array(xs)
    x = np.concatenate([x, -x])
    out = {}
    for fn in (2, 3):
        o = np.zeros_like(x)
        L.hyko_dm_eval(fn, x.ctypes.data_as(pd), np.zeros_like(x).ctypes.data_as(pd), o.ctypes.data_as(pd),
                       ctypes.c_uint64(len(x)))
        out[fn] = o
    worst = 0.0
    for i, xi in enumerate(x):
        xm = mpmath.mpf(float(xi))
        for fn, f in ((2, mpmath.sin), (3, mpmath.cos)):
            ref = f(xm)
            got = out[fn][i]
            sp = np.spacing(abs(float(ref))) if ref != 0 else np.spacing(0.0)
            err = float(abs(mpmath.mpf(float(got)) - ref)) / sp
            worst = max(worst, err)
            assert err <= 2.0, (fn, float(xi), got, float(ref), err)
    # single precision: the float functions go through the exact reduction from |x| = 2^16
    xf = np.ldexp(rng.uniform(1.0, 2.0, 400), rng.integers(16, 128, 400)).astype(np.float32).astype(np.float64)
    for fn, f in ((8, mpmath.sin), (9, mpmath.cos)):
        o = np.zeros_like(xf)
        L.hyko_dm_eval(fn, xf.ctypes.data_as(pd), np.zeros_like(xf).ctypes.data_as(pd), o.ctypes.data_as(pd),
                       ctypes.c_uint64(len(xf)))
        for xi, got in zip(xf, o):
            ref = float(f(mpmath.mpf(float(xi))))
            assert abs(got - ref) <= 1.01 * np.spacing(np.float32(abs(ref))), (fn, xi, got, ref)
