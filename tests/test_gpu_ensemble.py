"""Ensemble propagations against serial propagations, as the reference tests
them (heyoka/_test_ensemble.py:13-178): bit-identical states, times,
propagate_res, grid output and continuous output."""

import numpy as np
import pytest
import torch

import hyk

pytestmark = pytest.mark.gpu


def pend():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, -9.8 * hyk.sin(x))]


@pytest.fixture(scope="module")
def setup(libhyk):
    assert torch.cuda.is_available()
    ta = hyk.taylor_adaptive_batch(pend(), [[0.0] * 4] * 2)
    ics = np.zeros((10, 2, 4))
    for i in range(10):
        ics[i, 0] = [0.05 + i / 100, 0.051 + i / 100, 0.052 + i / 100, 0.053 + i / 100.0]
        ics[i, 1] = [0.025 + i / 100, 0.026 + i / 100, 0.027 + i / 100, 0.028 + i / 100.0]
    return ta, ics


@pytest.mark.parametrize("algo", ["thread", "process"])
def test_until_and_for(setup, algo):
    ta, ics = setup

    def gen(t, idx):
        t.set_time(0.0)
        t.state[:] = ics[idx]
        return t

    kw = {"max_workers": 8} if algo == "thread" else {"max_workers": 8, "chunksize": 3}
    ret = hyk.ensemble_propagate_until_batch(ta, 20.0, 10, gen, algorithm=algo, **kw)
    assert len(ret) == 10
    for i in range(10):
        ta.set_time(0.0)
        ta.state[:] = ics[i]
        ta.propagate_until(20.0)
        assert np.all(ret[i][0].time == 20.0)
        assert np.all(ta.state == ret[i][0].state)
        assert ret[i][1] is None
        assert ta.propagate_res == ret[i][0].propagate_res

    ret = hyk.ensemble_propagate_until_batch(ta, 20.0, 10, gen, algorithm=algo, c_output=True, **kw)
    for i in range(10):
        ta.set_time(0.0)
        ta.state[:] = ics[i]
        loc = ta.propagate_until(20.0, c_output=True)
        assert np.all(ta.state == ret[i][0].state)
        assert ret[i][1] is not None
        assert np.all(loc[0](5.0) == ret[i][1](5.0))

    def gen10(t, idx):
        t.set_time(10.0)
        t.state[:] = ics[idx]
        return t

    ret = hyk.ensemble_propagate_for_batch(ta, 20.0, 10, gen10, algorithm=algo, **kw)
    for i in range(10):
        ta.set_time(10.0)
        ta.state[:] = ics[i]
        ta.propagate_for(20.0)
        assert np.all(ret[i][0].time == 30.0)
        assert np.all(ta.state == ret[i][0].state)
        assert ta.propagate_res == ret[i][0].propagate_res


def test_grid(setup):
    ta, ics = setup
    grid = np.linspace(0.0, 20.0, 80)
    splat = np.repeat(grid, 4).reshape(-1, 4)

    def gen(t, idx):
        t.set_time(0.0)
        t.state[:] = ics[idx]
        return t

    ret = hyk.ensemble_propagate_grid_batch(ta, grid, 10, gen)
    for i in range(10):
        ta.set_time(0.0)
        ta.state[:] = ics[i]
        loc = ta.propagate_grid(splat)
        assert np.all(loc[1] == ret[i][2])
        assert np.all(ta.state == ret[i][0].state)
        assert ta.propagate_res == ret[i][0].propagate_res


def test_errors(setup):
    ta, _ = setup

    def gen(t, idx):
        return t

    with pytest.raises(TypeError, match="The n_iter parameter must be an integer"):
        hyk.ensemble_propagate_until(ta, 20.0, "a", gen)
    with pytest.raises(ValueError, match="The n_iter parameter must be non-negative"):
        hyk.ensemble_propagate_until(ta, 20.0, -1, gen)
    with pytest.raises(TypeError, match="must be a scalar, not an iterable object"):
        hyk.ensemble_propagate_until(ta, [20.0], 10, gen)
    with pytest.raises(TypeError, match="must be a scalar, not an iterable object"):
        hyk.ensemble_propagate_for(ta, [20.0], 10, gen)
    with pytest.raises(ValueError, match="one-dimensional, but instead it has 2 dimensions"):
        hyk.ensemble_propagate_grid(ta, [[20.0, 20.0]], 10, gen)
    with pytest.raises(TypeError, match='"max_delta_t" argument must be a scalar'):
        hyk.ensemble_propagate_until(ta, 20.0, 10, gen, max_delta_t=[10])
    with pytest.raises(TypeError):
        hyk.ensemble_propagate_until(ta, 20.0, 10, gen, chunksize=1)
    with pytest.raises(ValueError, match="parallelisation algorithm must be one of"):
        hyk.ensemble_propagate_until(ta, 20.0, 10, gen, algorithm="foo")
    assert hyk.ensemble_propagate_until(ta, 20.0, 0, gen) == []


def test_ensemble_with_events_matches_serial():
    """An ensemble with events runs every iteration's callbacks (deep-copied
    per iteration) on that iteration's integrator and lane; a terminal
    callback that changes the state (a bounce) and resumes the lane acts on
    the combined batch.  States, times and callback records equal those of
    the iterations run one by one."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, hyk.expression(-9.8))]  # a ball falling on the floor x = 0

    class Rec:
        def __init__(self):
            self.hits = []

        def __call__(self, ta, t, d_sgn, bidx):
            self.hits.append((bidx, t, d_sgn))

    class Bounce:
        def __init__(self):
            self.n = 0

        def __call__(self, ta, d_sgn, bidx):
            self.n += 1
            ta.state[1, bidx] = -0.8 * float(np.asarray(ta.state)[1, bidx])
            return True

    def make():
        return hyk.taylor_adaptive_batch(sys_, [[1.0] * 3, [0.0] * 3],
                                         nt_events=[hyk.nt_event_batch(v, Rec())],
                                         t_events=[hyk.t_event_batch(x, callback=Bounce(),
                                                                     direction=hyk.event_direction.negative)])

    heights = np.array([[1.0, 1.5, 2.0], [0.5, 0.7, 0.9], [1.2, 0.3, 2.5], [0.8, 1.1, 1.4]])

    def gen(t, i):
        t.set_time(0.0)
        t.state[:] = np.stack([heights[i], np.zeros(3)])
        return t

    ret = hyk.ensemble_propagate_until(make(), 3.0, 4, gen)
    for i, (ti, _, _) in enumerate(ret):
        ref = gen(make(), i)
        ref.propagate_until(3.0)
        assert np.array_equal(np.asarray(ti.state), np.asarray(ref.state)), i
        assert np.array_equal(ti.time, ref.time)
        assert ti.t_events[0].callback.n == ref.t_events[0].callback.n > 0
        # per lane in chronological order; the interleaving of lanes follows the kernel launches
        assert sorted(ti.nt_events[0].callback.hits) == sorted(ref.nt_events[0].callback.hits)
        for lane in range(3):
            ts = [t for b, t, _ in ti.nt_events[0].callback.hits if b == lane]
            assert ts == sorted(ts)


@pytest.mark.parametrize("devices", [[0], [0, 0], [0, 0, 0]])
@pytest.mark.parametrize("tp", ["until", "grid"])
def test_devices_equal_single_device(setup, devices, tp):
    """ensemble_propagate_* with devices= (iteration ranges per GPU, one host
    thread per GPU, results in iteration order): on one GPU named several
    times, bit-identical to the single-device ensemble."""
    ta, ics = setup

    def gen(t, idx):
        t.set_time(0.0)
        t.state[:] = ics[idx]
        return t

    if tp == "until":
        a = hyk.ensemble_propagate_until_batch(ta, 15.0, 10, gen)
        b = hyk.ensemble_propagate_until_batch(ta, 15.0, 10, gen, devices=devices)
    else:
        grid = np.linspace(0.0, 15.0, 7)
        a = hyk.ensemble_propagate_grid_batch(ta, grid, 10, gen)
        b = hyk.ensemble_propagate_grid_batch(ta, grid, 10, gen, devices=devices)
        for x, y in zip(a, b):
            assert np.array_equal(x[2], y[2])
    assert len(b) == 10
    for i, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(np.asarray(x[0].state), np.asarray(y[0].state)), i
        assert np.all(y[0].time == 15.0)
        assert x[0].propagate_res == y[0].propagate_res
