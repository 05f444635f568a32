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
