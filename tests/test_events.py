"""Events on the CPU: the event classes (the reference's tests of
nt_event_batch / t_event_batch, heyoka/test.py:410-690), the kernels' root
finder (hyk_events.h, through the oracle) and the oracle's propagation with
events against analytic solutions and the reference's event-count test
(heyoka/test.py:693-760)."""

import gc
import math
import pickle
from copy import copy, deepcopy

import numpy as np
import pytest

import hyk
from hyk import event_direction, nt_event_batch, t_event_batch


def test_event_classes_like_the_reference():
    x, v = hyk.make_vars("x", "v")
    ev = nt_event_batch(x + v, lambda _: _)
    assert " non-terminal" in repr(ev) and "(x + v)" in repr(ev) and "event_direction::any" in repr(ev)
    assert ev.expression == x + v and ev.direction == event_direction.any and ev.callback is not None
    ev = nt_event_batch(ex=x + v, callback=lambda _: _, direction=event_direction.negative)
    assert "event_direction::negative" in repr(ev)

    class local_cb:
        def __init__(self):
            self.n = 0

        def __call__(self, ta, t, d_sgn):
            self.n += 1

    lcb = local_cb()
    ev = nt_event_batch(ex=x + v, callback=lcb, direction=event_direction.negative)
    cb = ev.callback
    cb(1, 2, 3)
    cb(1, 2, 3)
    assert ev.callback.n == 2 and id(lcb) != id(ev.callback)
    with pytest.raises(ValueError, match="10 is not a valid event_direction"):
        nt_event_batch(ex=x + v, callback=lambda _: _, direction=event_direction(10))
    with pytest.raises(TypeError, match="cannot be used as an event callback because it is not callable"):
        nt_event_batch(ex=x + v, callback=3)
    with pytest.raises(TypeError, match="cannot be used as an event callback because it is not callable"):
        nt_event_batch(ex=x + v, callback=None)
    with pytest.raises(TypeError, match="is not recognized/supported"):
        nt_event_batch(x + v, lambda _: _, fp_type=str)

    ev = t_event_batch(x + v)
    r = repr(ev)
    assert " terminal" in r and ": no" in r and "auto" in r and ev.cooldown == -1.0 and ev.callback is None
    ev = t_event_batch(x + v, direction=event_direction.positive, cooldown=3.0, callback=lambda _: _)
    r = repr(ev)
    assert "event_direction::positive" in r and ": yes" in r and "3" in r and ev.cooldown == 3.0
    with pytest.raises(TypeError, match="not callable"):
        t_event_batch(x + v, callback=3)
    with pytest.raises(TypeError, match="is not recognized/supported"):
        t_event_batch(x + v, fp_type=list)


def test_event_pickle_copy_and_callback_lifetime():
    x, v = hyk.make_vars("x", "v")
    pytest.importorskip("cloudpickle")
    ev = nt_event_batch(ex=x + v, callback=lambda _: _, direction=event_direction.negative)
    ev = pickle.loads(pickle.dumps(ev))
    assert "event_direction::negative" in repr(ev)
    ev.foo = "hello world"
    ev = pickle.loads(pickle.dumps(ev))
    assert ev.foo == "hello world"

    class foo:
        pass

    ev.bar = foo()
    assert id(ev.bar) == id(copy(ev).bar)
    assert id(ev.bar) != id(deepcopy(ev).bar)
    ev = t_event_batch(x + v, direction=event_direction.positive, cooldown=3.0)
    ev = pickle.loads(pickle.dumps(ev))
    assert ": no" in repr(ev) and "3" in repr(ev)

    class counter:
        def __init__(self):
            self.n = 0

        def __call__(self, ta, d_sgn):
            self.n += 1

    ev = t_event_batch(ex=x + v, callback=counter(), direction=event_direction.negative)
    out_cb = ev.callback
    del ev
    gc.collect()
    out_cb(1, 2)
    assert out_cb.n == 1


def test_root_finder_against_numpy(oracle):
    rng = np.random.default_rng(1)
    for _ in range(200):
        k = int(rng.integers(1, 5))
        roots = np.sort(rng.uniform(0.02, 0.98, k))
        if k > 1 and np.min(np.diff(roots)) < 1e-3:
            continue
        c = np.polynomial.polynomial.polyfromroots(roots) * rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-3, 3)
        c = np.concatenate([c, rng.normal(0, 1e-30, 12)])  # degree padding with negligible terms
        h = rng.uniform(0.1, 3.0) * rng.choice([-1.0, 1.0])
        g = c / h ** np.arange(len(c))  # g_n h^n = c_n: the polynomial in s has the chosen roots
        rs, sg, n = oracle.ev_find(g, h)
        assert n == k and np.allclose(rs, roots, atol=1e-9)
        dq = np.polynomial.polynomial.polyval(roots, np.polynomial.polynomial.polyder(c))
        assert np.array_equal(sg, (np.sign(dq) * np.sign(h)).astype(np.int32))
        # direction filter and window
        rs_p, sg_p, _ = oracle.ev_find(g, h, direction=1)
        assert np.all(sg_p == 1) and len(rs_p) == int(np.sum(sg == 1))
        rs_w, _, _ = oracle.ev_find(g, h, s_lo=roots[0] + 1e-7)
        assert len(rs_w) == k - 1
    # close roots (the reference's v*v - 1e-10 event: two roots 2e-5 apart)
    c = np.polynomial.polynomial.polyfromroots([0.5 - 1e-5, 0.5 + 1e-5])
    c = np.concatenate([c, np.zeros(18)])
    rs, sg, n = oracle.ev_find(c, 1.0)
    assert n == 2 and np.allclose(rs, [0.5 - 1e-5, 0.5 + 1e-5], atol=1e-12) and list(sg) == [-1, 1]
    # no root
    assert oracle.ev_find(np.concatenate([[1.0, 0.1], np.zeros(19)]), 1.0)[2] == 0


def test_oracle_events_harmonic_oscillator(oracle):
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -x)]
    st = np.array([[1.0, 2.0, -0.5], [0.0, 0.0, 0.0]])
    r = oracle.propagate_ev(sys_, [(x, False, 0, -1.0), (v, False, 1, -1.0)], st, 20.0, order=20)
    for lane in range(3):
        m = r["rec_lane"] == lane
        t = r["rec_t_hi"][m]
        info = r["rec_info"][m]
        tx = np.sort(t[(info >> 2) == 0])
        assert np.allclose(tx, [math.pi / 2 + k * math.pi for k in range(len(tx))], atol=1e-13) and len(tx) == 6
        # v = -A sin t increases through 0 where sin t goes from + to -: t = (2k+1) pi for A > 0
        tv = t[(info >> 2) == 1]
        A = st[0, lane]
        want = [k * math.pi for k in range(1, 7) if np.sign(-A * math.cos(k * math.pi)) > 0]
        assert np.allclose(np.sort(tv), want, atol=1e-13)
    # terminal: stops at the first root, direction and cooldown respected
    r = oracle.propagate_ev(sys_, [(x, True, 1, -1.0)], st, 20.0, order=20)
    assert list(r["outcome"]) == [-1, -1, -1]  # a propagation stopped by terminal event k reports -k - 1
    assert np.allclose(r["t_hi"], [1.5 * math.pi, 1.5 * math.pi, 0.5 * math.pi], atol=1e-13)
    assert list(r["ev_sign"]) == [1, 1, 1]
    r2 = oracle.propagate_ev(sys_, [(x, True, 1, -1.0)], r["state"], 20.0, order=20, time=r["t_hi"],
                             ev_last=r["ev_last"])
    assert np.allclose(r2["t_hi"], r["t_hi"] + 2 * math.pi, atol=1e-12)


def test_oracle_reference_event_counts(oracle):
    """heyoka/test.py:705-760: pendulum, two lanes, non-terminal events
    v*v - 1e-10 and v to t = 4: 12 roots per lane in all (the reference's
    counter is shared by both callbacks), in the pattern (v*v-1e-10, v,
    v*v-1e-10) around each of the 4 turning points."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    r = oracle.propagate_ev(sys_, [(v * v - 1e-10, False, 0, -1.0), (v, False, 0, -1.0)],
                            np.array([[0.0, 0.001], [0.25, 0.2501]]), 4.0, order=20)
    assert list(r["outcome"]) == [int(hyk.taylor_outcome.time_limit)] * 2
    for lane in range(2):
        m = r["rec_lane"] == lane
        order = np.argsort(r["rec_t_hi"][m], kind="stable")
        ks = (r["rec_info"][m] >> 2)[order]
        assert len(ks) == 12
        assert list(ks) == [0, 1, 0] * 4
        t = np.sort(r["rec_t_hi"][m])
        assert np.all(np.diff(t) > 0)


def test_oracle_events_harmonic_oscillator_float32(oracle):
    """The float32 event path (root finder and event bookkeeping in single
    precision): roots of x and v of the harmonic oscillator at the analytic
    times, to single-precision accuracy; terminal event with the automatic
    cooldown of the float integrator."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -x)]
    st = np.array([[1.0, 2.0, -0.5], [0.0, 0.0, 0.0]])
    r = oracle.propagate_ev(sys_, [(x, False, 0, -1.0), (v, False, 1, -1.0)], st, 20.0, order=9, prec=2)
    for lane in range(3):
        m = r["rec_lane"] == lane
        t = r["rec_t_hi"][m] + r["rec_t_lo"][m]
        info = r["rec_info"][m]
        tx = np.sort(t[(info >> 2) == 0])
        assert len(tx) == 6 and np.allclose(tx, [math.pi / 2 + k * math.pi for k in range(6)], atol=2e-5)
        assert np.all(r["rec_t_hi"][m] == r["rec_t_hi"][m].astype(np.float32))
    r = oracle.propagate_ev(sys_, [(x, True, 1, -1.0)], st, 20.0, order=9, prec=2)
    assert list(r["outcome"]) == [-1, -1, -1] and list(r["ev_sign"]) == [1, 1, 1]
    assert np.allclose(r["t_hi"], [1.5 * math.pi, 1.5 * math.pi, 0.5 * math.pi], atol=2e-5)
    r2 = oracle.propagate_ev(sys_, [(x, True, 1, -1.0)], r["state"], 20.0, order=9, prec=2, time=r["t_hi"],
                             time_lo=r["t_lo"], ev_last=r["ev_last"])
    assert np.allclose(r2["t_hi"], r["t_hi"] + 2 * math.pi, atol=5e-5)
