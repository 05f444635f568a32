"""Step callbacks of propagate_until / propagate_for / propagate_grid: the
reference's behaviour (heyoka/_test_batch_integrator.py test_propagate_for,
callback parts; heyoka/step_cb_utils.cpp) in both precisions, and results
identical to a propagation without callback when every call returns True."""

import numpy as np
import pytest
import torch

import hyk

pytestmark = pytest.mark.gpu


def _pend():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, -9.8 * hyk.sin(x))]


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_reference_callback_behaviour(fp_t):
    ic = np.array([[0.0, 0.1, 0.2, 0.3], [0.25, 0.26, 0.27, 0.28]], dtype=fp_t)
    ta = hyk.taylor_adaptive_batch(_pend(), ic, fp_type=fp_t)

    def cb(ta):
        if hasattr(ta, "counter"):
            ta.counter += 1
        else:
            ta.counter = 0
        return True

    ta.propagate_for(fp_t(10.0), callback=cb)
    assert ta.counter > 0

    class cb_id:
        def __call__(_, ta):
            assert id(_) == _.orig_id
            return True

    inst = cb_id()
    inst.orig_id = id(inst)
    _, ret = ta.propagate_for(fp_t(10.0), callback=inst)
    assert ret is inst

    with pytest.raises(TypeError, match="cannot be used as a step callback because it is not callable"):
        ta.set_time(fp_t(0.0))
        ta.state[:] = ic
        ta.propagate_for(fp_t(10.0), callback="hello world")

    class broken_cb:
        def __call__(self, ta):
            return []

    with pytest.raises(TypeError, match="The call operator of a step callback is expected to return a boolean, "
                                        "but a value of type"):
        ta.set_time(fp_t(0.0))
        ta.state[:] = ic
        ta.propagate_for(fp_t(10.0), callback=broken_cb())

    class cb_hook:
        def __call__(_, ta):
            return True

        def pre_hook(self, ta):
            ta.foo = True

    ta.set_time(fp_t(0.0))
    ta.state[:] = ic
    ta.propagate_for(fp_t(10.0), callback=cb_hook())
    assert ta.foo
    delattr(ta, "foo")


def test_callback_results_and_stop():
    rng = np.random.default_rng(3)
    st = np.stack([rng.uniform(-1, 1, 300), rng.uniform(-0.5, 0.5, 300)])
    a = hyk.taylor_adaptive_batch(_pend(), st)
    b = hyk.taylor_adaptive_batch(_pend(), st)
    calls = []

    def count(ta):
        calls.append(float(ta.time.max()))
        return True

    a.propagate_until(20.0, callback=count)
    b.propagate_until(20.0)
    # one call per batch step, the same bits as without a callback
    assert len(calls) == int(b.propagate_res_tensors["n_iter"].max().item())
    assert torch.equal(a.state, b.state) and a.propagate_res == b.propagate_res
    assert np.all(np.diff(calls) >= 0)

    # a callback returning False stops every lane with cb_stop
    c = hyk.taylor_adaptive_batch(_pend(), st)
    n = [0]

    def stop_after_5(ta):
        n[0] += 1
        return n[0] < 5

    c.propagate_until(20.0, callback=stop_after_5)
    assert n[0] == 5
    assert all(r[0] == hyk.taylor_outcome.cb_stop and r[3] == 5 for r in c.propagate_res)
    assert np.all(c.time < 20.0)
    # and the propagation resumes from there (the final step is clamped by
    # the remaining time recomputed at the restart, so only to rounding)
    c.propagate_until(20.0)
    assert torch.allclose(c.state, b.state, rtol=1e-12, atol=1e-14)

    # a list of callbacks: all are called after each step
    seen = [0, 0]

    def c0(ta):
        seen[0] += 1
        return True

    def c1(ta):
        seen[1] += 1
        return True

    d = hyk.taylor_adaptive_batch(_pend(), st)
    d.propagate_until(5.0, callback=[c0, c1])
    assert seen[0] == seen[1] > 0

    # propagate_grid returns the callback first
    e = hyk.taylor_adaptive_batch(_pend(), st)
    grid = np.repeat(np.linspace(0.0, 5.0, 11).reshape(-1, 1), 300, axis=1)
    ret, out = e.propagate_grid(grid, callback=c0)
    assert ret is c0 and out.shape == (11, 2, 300)
    f = hyk.taylor_adaptive_batch(_pend(), st)
    _, out2 = f.propagate_grid(grid)
    assert np.array_equal(out, out2)


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_reference_step_callback_lists_and_angle_reducer(fp_t):
    """heyoka/_test_batch_integrator.py test_step_callback."""
    from hyk.callback import angle_reducer

    x, v = hyk.make_vars("x", "v")

    class cb_hook:
        def __call__(_, ta):
            return True

        def pre_hook(self, ta):
            ta.foo = True

    ta = hyk.taylor_adaptive_batch([(x, v), (v, -9.8 * hyk.sin(x))],
                                   [[fp_t(0.0), fp_t(0.01)], [fp_t(10.0), fp_t(10.01)]], fp_type=fp_t)
    cb1, cb2 = cb_hook(), cb_hook()
    res = ta.propagate_for(fp_t(10.0), callback=[cb1, cb2])
    assert isinstance(res[1], list) and res[1][0] is cb1 and res[1][1] is cb2
    assert hasattr(ta, "foo")
    res = ta.propagate_until(fp_t(20.0), callback=[cb1, angle_reducer([x]), cb2])
    assert isinstance(res[1][1], angle_reducer) and res[1][0] is cb1 and res[1][2] is cb2
    st = np.asarray(ta.state)
    assert 0 <= st[0, 0] < 6.29 and 0 <= st[0, 1] < 6.29
    res = ta.propagate_grid([[fp_t(20.0), fp_t(20.0)], [fp_t(30.0), fp_t(30.1)]], callback=cb1)
    assert res[0] is cb1
    res = ta.propagate_for(fp_t(10.0), callback=angle_reducer([x]))
    assert isinstance(res[1], angle_reducer)
    st = np.asarray(ta.state)
    assert 0 <= st[0, 0] < 6.29 and 0 <= st[0, 1] < 6.29


def test_ensemble_callbacks_deep_copied():
    """heyoka/_test_ensemble.py: the callbacks of an ensemble propagation are
    deep copies, one per iteration, returned in the results; a callback that
    stops its iteration stops only that iteration."""
    from hyk.callback import angle_reducer

    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    rng = np.random.default_rng(1)
    ics = [np.stack([rng.uniform(-1, 1, 2), rng.uniform(-0.5, 0.5, 2)]) for _ in range(10)]
    ta = hyk.taylor_adaptive_batch(sys_, ics[0])

    class step_cb:
        def __call__(_, ta):
            assert id(_) != _.orig_id
            return True

    cb = step_cb()
    cb.orig_id = id(cb)

    def gen(ta, idx):
        ta.set_time(0.0)
        ta.state[:] = ics[idx]
        return ta

    ret = hyk.ensemble_propagate_for_batch(ta, 20.0, 10, gen, algorithm="thread", max_workers=8, callback=cb)
    for r in ret:
        assert isinstance(r[2], step_cb)
    ret = hyk.ensemble_propagate_for_batch(ta, 20.0, 10, gen, callback=[cb, angle_reducer([x])])
    for r in ret:
        assert isinstance(r[2], list) and len(r[2]) == 2
        assert isinstance(r[2][0], step_cb) and isinstance(r[2][1], angle_reducer)

    class stopper:
        def __init__(self):
            self.n = 0

        def __call__(self, ta):
            self.n += 1
            return not (ta.stop_me and self.n >= 3)

    def gen2(ta, idx):
        ta.set_time(0.0)
        ta.state[:] = ics[idx]
        ta.stop_me = idx == 4
        return ta

    ret = hyk.ensemble_propagate_until(ta, 20.0, 10, gen2, callback=stopper())
    for i, r in enumerate(ret):
        if i == 4:
            assert all(o[0] == hyk.taylor_outcome.cb_stop for o in r[0].propagate_res) and r[2].n == 3
        else:
            assert all(o[0] == hyk.taylor_outcome.time_limit for o in r[0].propagate_res)
            assert np.all(r[0].time == 20.0) and r[2].n > 3
