"""The scalar integrator ``taylor_adaptive`` (one lane) and ensembles of it:
the reference's scalar API (heyoka/taylor_expose_integrator.cpp:90-420) and
its ensemble tests (heyoka/_test_ensemble.py test_scalar), and the
batch/scalar agreement of heyoka/_test_batch_integrator.py
test_propagate_grid (bit for bit here: a lane's arithmetic does not depend
on its batch)."""

import pickle
from copy import deepcopy

import numpy as np
import pytest

import hyk

pytestmark = pytest.mark.gpu


def _sys():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, -9.8 * hyk.sin(x))]


def test_scalar_api(oracle):
    ta = hyk.taylor_adaptive(_sys(), [0.05, 0.025])
    assert ta.order == 20 and ta.dim == 2 and ta.time == 0.0 and ta.state.shape == (2,)
    oc, h = ta.step()
    assert oc == hyk.taylor_outcome.success and h > 0
    o = oracle.Oracle(_sys(), np.array([[0.05], [0.025]]), order=20, mode=1)
    _, oh = o.step()
    assert h == oh[0] and np.array_equal(np.asarray(ta.state), o.state[:, 0])
    oc, h = ta.step(0.01)
    assert oc == hyk.taylor_outcome.time_limit and h == 0.01
    oc, h = ta.step_backward()
    assert h < 0
    ta.time = 0.0
    ta.state[:] = [0.05, 0.025]
    r = ta.propagate_until(20.0)
    assert len(r) == 6 and r[0] == hyk.taylor_outcome.time_limit and r[4] is None and r[5] is None
    assert ta.time == 20.0
    ta.time = 0.0
    ta.state[:] = [0.05, 0.025]
    r = ta.propagate_for(5.0, c_output=True)
    c = r[4]
    assert isinstance(c, hyk.continuous_output) and c.bounds == (0.0, 5.0)
    assert np.allclose(c(5.0), np.asarray(ta.state), rtol=1e-14, atol=1e-15)
    assert c(np.array([1.0, 2.0, 3.0])).shape == (3, 2)
    d = ta.update_d_output(5.0)
    assert d.shape == (2,)
    ta.dtime = (1.0, 0.5)
    assert ta.dtime == (1.5, 0.0)
    ta.time = 0.0
    ta.state[:] = [0.05, 0.025]
    res = ta.propagate_grid(np.linspace(0.0, 10.0, 11))
    assert len(res) == 6 and res[4] is None and res[5].shape == (11, 2)
    ta.foo = 1
    t2 = deepcopy(ta)
    assert t2.foo == 1 and np.array_equal(np.asarray(t2.state), np.asarray(ta.state))
    t3 = pickle.loads(pickle.dumps(ta))
    assert t3.time == ta.time and np.array_equal(np.asarray(t3.state), np.asarray(ta.state))

    calls = []

    def cb(ta_):
        assert ta_ is ta
        calls.append(ta_.time)
        return True

    ta.time = 0.0
    r = ta.propagate_until(3.0, callback=cb)
    assert r[5] is cb and len(calls) == r[3]


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_batch_scalar_grid_agreement(fp_t):
    x, v = hyk.make_vars("x", "v")
    eqns = [(x, v), (v, -9.8 * hyk.sin(x))]
    x_ic = np.array([0.06, 0.07, 0.08, 0.09], dtype=fp_t)
    v_ic = np.array([0.025, 0.026, 0.027, 0.028], dtype=fp_t)
    ta = hyk.taylor_adaptive_batch(eqns, [x_ic, v_ic], fp_type=fp_t)
    tas = [hyk.taylor_adaptive(eqns, [x0, v0], fp_type=fp_t) for x0, v0 in zip(x_ic, v_ic)]
    grid = np.array([[-0.1, -0.2, -0.3, -0.4], [0.01, 0.02, 0.03, 0.9], [1.0, 1.1, 1.2, 1.3],
                     [11.0, 11.1, 11.2, 11.3]], dtype=fp_t)
    ta.propagate_until(grid[0, :])
    bres = ta.propagate_grid(grid)
    assert bres[0] is None
    for i, s in enumerate(tas):
        s.propagate_until(grid[0, i])
        sres = s.propagate_grid(grid[:, i])
        assert np.array_equal(sres[5], bres[1][:, :, i])


def test_scalar_ensembles():
    """heyoka/_test_ensemble.py test_scalar (thread algorithm)."""
    ta = hyk.taylor_adaptive(_sys(), [0.0] * 2)
    ics = np.array([[0.05, 0.025]] * 10)
    for i in range(10):
        ics[i] += i / 100.0

    def gen(ta, idx):
        ta.time = 0.0
        ta.state[:] = ics[idx]
        return ta

    ret = hyk.ensemble_propagate_until(ta, 20.0, 10, gen, algorithm="thread", max_workers=8)
    assert len(ret) == 10 and all(r[1] == hyk.taylor_outcome.time_limit for r in ret)
    for i in range(10):
        ta.time = 0.0
        ta.state[:] = ics[i]
        loc = ta.propagate_until(20.0)
        assert ret[i][0].time == 20.0
        assert np.all(np.asarray(ta.state) == np.asarray(ret[i][0].state))
        assert loc == ret[i][1:]
    ret = hyk.ensemble_propagate_until(ta, 20.0, 10, gen, c_output=True)
    for i in range(10):
        ta.time = 0.0
        ta.state[:] = ics[i]
        loc = ta.propagate_until(20.0, c_output=True)
        assert loc[:-2] == ret[i][1:-2]
        assert np.all(loc[-2](5.0) == ret[i][-2](5.0))

    def gen_for(ta, idx):
        ta.time = 10.0
        ta.state[:] = ics[idx]
        return ta

    ret = hyk.ensemble_propagate_for(ta, 20.0, 10, gen_for)
    for i in range(10):
        ta.time = 10.0
        ta.state[:] = ics[i]
        loc = ta.propagate_for(20.0)
        assert ret[i][0].time == 30.0 and loc == ret[i][1:]

    grid = np.linspace(0.0, 20.0, 80)
    ret = hyk.ensemble_propagate_grid(ta, grid, 10, gen)
    for i in range(10):
        ta.time = 0.0
        ta.state[:] = ics[i]
        loc = ta.propagate_grid(grid)
        assert loc[:4] == ret[i][1:5] and np.array_equal(loc[5], ret[i][6])

    class step_cb:
        def __call__(_, ta):
            assert id(_) != _.orig_id
            ta.seen = True
            return True

    cb = step_cb()
    cb.orig_id = id(cb)
    ret = hyk.ensemble_propagate_until(ta, 20.0, 10, gen, callback=cb)
    for r in ret:
        assert isinstance(r[-1], step_cb) and r[0].seen


def test_scalar_events():
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    roots = []

    def cb(ta, t, d_sgn):
        assert isinstance(ta, hyk.taylor_adaptive)
        roots.append((t, d_sgn))

    ta = hyk.taylor_adaptive(sys_, [0.05, 0.025], nt_events=[hyk.nt_event(v, cb)])
    assert ta.with_events and len(ta.nt_events) == 1
    assert id(ta.nt_events[0].callback) == id(ta.nt_events[0].callback)
    r = ta.propagate_until(10.0)
    assert r[0] == hyk.taylor_outcome.time_limit
    # the same roots as the batch integrator's (one lane)
    broots = []
    tb = hyk.taylor_adaptive_batch(sys_, [[0.05], [0.025]],
                                   nt_events=[hyk.nt_event_batch(v, lambda ta, t, d, b: broots.append((t, d)))])
    tb.propagate_until(10.0)
    assert roots == broots and len(roots) > 5
    # the callback objects belong to the integrator: a deep copy has its own
    # (functions deep-copy to themselves; a callable object does not)

    class cbk:
        def __call__(self, ta, t, d_sgn):
            pass

    ta3 = hyk.taylor_adaptive(sys_, [0.05, 0.025], nt_events=[hyk.nt_event(v, cbk())])
    t2 = deepcopy(ta3)
    assert id(t2.nt_events[0].callback) != id(ta3.nt_events[0].callback)

    class stop:
        def __init__(self):
            self.n = 0

        def __call__(self, ta, d_sgn):
            self.n += 1
            return False

    ta = hyk.taylor_adaptive(sys_, [0.05, 0.025], t_events=[hyk.t_event(v, callback=stop(),
                                                                          direction=hyk.event_direction.negative)])
    r = ta.propagate_until(10.0)
    assert int(r[0]) == -1 and ta.time < 10.0
    assert ta.t_events[0].callback.n == 1
    assert ta.te_cooldowns[0] is not None
    ta.reset_cooldowns()
    assert ta.te_cooldowns[0] is None
    oc, h = ta.step()
    assert oc == hyk.taylor_outcome.success or int(oc) >= 0


def test_scalar_ensemble_with_events():
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]

    class counter:
        def __init__(self):
            self.n = 0

        def __call__(self, ta, t, d_sgn):
            assert isinstance(ta, hyk.taylor_adaptive)
            self.n += 1
            ta.seen = True

    ta = hyk.taylor_adaptive(sys_, [0.05, 0.025], nt_events=[hyk.nt_event(v, counter())])

    def gen(ta, i):
        ta.time = 0.0
        ta.state[:] = [0.05 + 0.01 * i, 0.025]
        return ta

    ret = hyk.ensemble_propagate_until(ta, 10.0, 6, gen)
    for r in ret:
        assert r[1] == hyk.taylor_outcome.time_limit
        assert r[0].nt_events[0].callback.n > 5 and r[0].seen


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_reference_scalar_nt_event_pattern(fp_t):
    """heyoka/test.py event_detection_test_case.test_scalar, non-terminal
    part: two events (v^2 - delta, v) on the pendulum, their roots in the
    order (v^2 - delta, v, v^2 - delta) around each turning point, twelve up
    to t = 4, each callback given the integrator itself."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    small = 1e-6 if fp_t == np.float32 else 1e-10
    state = {"n": 0, "t": fp_t(0), "id": None}

    def cb0(ta, t, d_sgn):
        assert t > state["t"] and state["n"] % 3 in (0, 2) and id(ta) == state["id"]
        state["n"] += 1
        state["t"] = t

    def cb1(ta, t, d_sgn):
        assert t > state["t"] and state["n"] % 3 == 1 and id(ta) == state["id"]
        state["n"] += 1
        state["t"] = t

    ta = hyk.taylor_adaptive(sys_, [fp_t(0), fp_t(0.25)], fp_type=fp_t,
                             nt_events=[hyk.nt_event(v * v - small, cb0, fp_type=fp_t),
                                        hyk.nt_event(v, cb1, fp_type=fp_t)])
    state["id"] = id(ta)
    assert ta.propagate_until(fp_t(4))[0] == hyk.taylor_outcome.time_limit
    assert state["n"] == 12


def test_reference_gil_bug_construction_error():
    """heyoka/test.py test_gil_bug: a failing construction with events raises
    ValueError cleanly."""
    x, v = hyk.make_vars("x", "v")

    class cb0:
        def __call__(self, ta, t, d_sgn):
            pass

    with pytest.raises(ValueError):
        hyk.taylor_adaptive([(x, v), (v, -9.8 * hyk.sin(x))], [0.0], nt_events=[hyk.nt_event(x, cb0())])


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_reference_c_output_batch_behaviour(fp_t):
    """heyoka/test.py c_output_test_case.test_batch, functional part."""
    from sys import getrefcount

    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    ic = np.array([[0.0, 0.01, 0.02, 0.03], [0.25, 0.26, 0.27, 0.28]], dtype=fp_t)
    ta = hyk.taylor_adaptive_batch(sys_, ic, fp_type=fp_t)
    scal = [hyk.taylor_adaptive(sys_, ic[:, i], fp_type=fp_t) for i in range(4)]
    final_tm = np.array([10.0, 10.4, 10.5, 11.0], dtype=fp_t)
    check_tm = np.array([0.1, 1.3, 5.6, 9.1], dtype=fp_t)
    c_out, cb = ta.propagate_until(final_tm)
    assert cb is None and c_out is None
    ta.state[:] = ic
    ta.set_time(fp_t(0))
    c_out, cb = ta.propagate_until(final_tm, c_output=True)
    assert cb is None and c_out is not None
    assert c_out(check_tm).shape == (2, 4)
    with pytest.raises(ValueError):
        c_out(check_tm)[0] = 0.5
    rc = getrefcount(c_out)
    tmp = c_out(check_tm)  # noqa: F841
    assert getrefcount(c_out) == rc + 1
    with pytest.raises(ValueError, match="the number of dimensions must be 1 or 2, but it is 3 instead"):
        c_out(np.zeros((1, 1, 1), dtype=fp_t))
    for n in (1, 0, 5):
        with pytest.raises(ValueError, match="the length must be 4 but it is {} instead".format(n)):
            c_out(np.zeros((n,), dtype=fp_t))
    eps = np.finfo(fp_t).eps * 10
    c_scal = [s.propagate_until(final_tm[i], c_output=True)[4] for i, s in enumerate(scal)]
    c_out(check_tm)
    for i in range(4):
        c_scal[i](check_tm[i])
        assert np.allclose(c_scal[i].output, c_out.output[:, i], rtol=eps, atol=eps)
    scal_res = c_out(fp_t(0.42)).copy()
    assert np.all(scal_res == c_out([fp_t(0.42)] * 4))
    nc = np.vstack([check_tm, np.zeros((4,), dtype=fp_t)]).T.flatten()[::2]
    c_out(nc)
    for i in range(4):
        assert np.allclose(c_scal[i].output, c_out.output[:, i], rtol=eps, atol=eps)
    with pytest.raises(ValueError, match="the number of columns must be 4 but it is 3 instead"):
        c_out(np.zeros((5, 3), dtype=fp_t))
    b = np.repeat(check_tm, 5, axis=0).reshape((4, 5)).T
    out_b = c_out(b)
    assert out_b.shape == (5, 2, 4)
    assert c_out(np.zeros((0, 4), dtype=fp_t)).shape == (0, 2, 4)
    assert c_out.times.shape == (c_out.n_steps + 1, 4) and np.all(np.isfinite(c_out.times))
    with pytest.raises(ValueError):
        c_out.times[0] = 0.5
    rc = getrefcount(c_out)
    tmp3 = c_out.times  # noqa: F841
    assert getrefcount(c_out) == rc + 1
    assert c_out.tcs.shape == (c_out.n_steps, 2, ta.order + 1, 4)


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_reference_c_output_scalar_behaviour(fp_t):
    """heyoka/test.py c_output_test_case.test_scalar (default construction,
    views that keep the object alive, shapes, errors, copies, pickling)."""
    import pickle
    from copy import copy, deepcopy
    from sys import getrefcount

    c_out = hyk.continuous_output_dbl() if fp_t is float else hyk.continuous_output_flt()
    with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output object"):
        c_out(fp_t(0))
    with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output object"):
        c_out(time=[fp_t(0), fp_t(0)])
    assert c_out(time=np.zeros((0,), dtype=fp_t)).shape == (0, 0)
    assert c_out.output is None and c_out.times is None and c_out.tcs is None
    for obj in (c_out, copy(c_out), deepcopy(c_out), pickle.loads(pickle.dumps(c_out))):
        with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output object"):
            obj.n_steps
        with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output object"):
            obj.bounds
        assert "forward" not in repr(obj) and obj.llvm_state.ir != ""

    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    ic = [fp_t(0), fp_t(0.25)]
    ta = hyk.taylor_adaptive(sys=sys_, state=ic, fp_type=fp_t)

    def reset():
        ta.state[:] = ic
        ta.time = fp_t(0)

    assert ta.propagate_until(fp_t(10))[4] is None
    reset()
    assert ta.propagate_until(fp_t(10), c_output=False)[4] is None
    reset()
    _, _, _, nsteps, c_out, cb = ta.propagate_until(fp_t(10), c_output=True)
    assert cb is None and c_out is not None
    assert c_out(fp_t(0.1)).shape == (2,)
    with pytest.raises(ValueError):
        c_out(fp_t(0.1))[0] = 0.5
    rc = getrefcount(c_out)
    tmp = c_out(fp_t(0.1))  # noqa: F841
    assert getrefcount(c_out) == rc + 1
    assert c_out(np.zeros((0,), dtype=fp_t)).shape == (0, 2)
    tmp = c_out([fp_t(0), fp_t(1), fp_t(2)])
    for i in range(3):
        assert np.all(c_out(fp_t(i)) == tmp[i])
    with pytest.raises(ValueError, match="Invalid time array passed to a continuous_output object: the number of "
                                         "dimensions must be 1, but it is 2 instead"):
        c_out([[fp_t(0)], [fp_t(1)], [fp_t(2)]])
    assert np.all(c_out.output == tmp[2])
    with pytest.raises(ValueError):
        c_out.output[0] = 0.5
    for name in ("output", "times", "tcs"):
        rc = getrefcount(c_out)
        held = getattr(c_out, name)  # noqa: F841
        assert getrefcount(c_out) == rc + 1
        del held
    assert c_out.times.shape == (nsteps + 1,)
    with pytest.raises(ValueError):
        c_out.times[0] = 0.5
    assert c_out.tcs.shape == (nsteps, 2, ta.order + 1) and np.all(np.isfinite(c_out.tcs))
    with pytest.raises(ValueError):
        c_out.tcs[0, 0, 0] = 0.5
    assert c_out.bounds == (0, 10) and c_out.n_steps > 0
    assert "forward" in repr(c_out) and c_out.llvm_state.ir != ""
    for c in (copy(c_out), deepcopy(c_out), pickle.loads(pickle.dumps(c_out))):
        assert c.tcs.shape == (nsteps, 2, ta.order + 1) and np.all(np.isfinite(c.tcs))
        with pytest.raises(ValueError):
            c.tcs[0, 0, 0] = 0.5

    class foo:
        pass

    c_copy = deepcopy(c_out)
    c_copy.bar = foo()
    assert id(c_copy.bar) == id(copy(c_copy).bar)
    assert id(c_copy.bar) != id(deepcopy(c_copy).bar)
    assert np.all(c_copy(fp_t(0.1)) == copy(c_copy)(fp_t(0.1)))
    assert np.all(c_copy(fp_t(0.1)) == deepcopy(c_copy)(fp_t(0.1)))
    c_out.foo = []
    c_out = pickle.loads(pickle.dumps(c_out))
    assert c_out.tcs.shape == (nsteps, 2, ta.order + 1) and c_out.foo == []


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_reference_c_output_batch_copies(fp_t):
    """heyoka/test.py c_output_test_case.test_batch: copies and pickles of a
    batch continuous output, with attributes added from Python."""
    import pickle
    from copy import copy, deepcopy

    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    ic = np.array([[0.0, 0.01, 0.02, 0.03], [0.25, 0.26, 0.27, 0.28]], dtype=fp_t)
    ta = hyk.taylor_adaptive_batch(sys_, ic, fp_type=fp_t)
    c_out = ta.propagate_until(np.array([10.0, 10.4, 10.5, 11.0], dtype=fp_t), c_output=True)[0]
    assert "forward" in repr(c_out)
    for c in (copy(c_out), deepcopy(c_out), pickle.loads(pickle.dumps(c_out))):
        assert c.tcs.shape == (c.n_steps, 2, ta.order + 1, 4) and c.llvm_state.ir != ""

    class foo:
        pass

    c_copy = deepcopy(c_out)
    c_copy.bar = foo()
    assert id(c_copy.bar) == id(copy(c_copy).bar)
    assert id(c_copy.bar) != id(deepcopy(c_copy).bar)
    assert np.all(c_copy(fp_t(0.1)) == copy(c_copy)(fp_t(0.1)))
    assert np.all(c_copy(fp_t(0.1)) == deepcopy(c_copy)(fp_t(0.1)))
    c_out.foo = []
    c_out = pickle.loads(pickle.dumps(c_out))
    assert c_out.tcs.shape == (c_out.n_steps, 2, ta.order + 1, 4) and c_out.foo == []
