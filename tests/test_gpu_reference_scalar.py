"""The reference's scalar-integrator tests, restated for the one-lane GPU
integrator (heyoka/_test_scalar_integrator.py test_dtime :85-115, test_copy
:117-143, test_basic :145-323, test_events :325-365, test_s11n :367-465,
test_step_callback :467-530), in single and double precision (long double and
real128 are not provided)."""

import pickle
from copy import copy, deepcopy

import numpy as np
import pytest

import hyk

pytestmark = pytest.mark.gpu

FP_TYPES = [np.float32, float]


def _pendulum():
    x, v = hyk.make_vars("x", "v")
    return x, v, [(x, v), (v, -9.8 * hyk.sin(x))]


def _cb0(ta, t, d_sgn):
    pass


class _Counter:
    def __call__(self, ta):
        if hasattr(ta, "counter"):
            ta.counter += 1
        else:
            ta.counter = 0
        return True


class _SameObject:
    def __call__(self, ta):
        assert id(self) == self.orig_id
        return True


class _Broken:
    def __call__(self, ta):
        return []


class _Hook:
    def __call__(self, ta):
        return True

    def pre_hook(self, ta):
        ta.foo = True


class _Stateful:
    def __init__(self):
        self.n = 0

    def __call__(self, ta, t, d_sgn):
        self.n = self.n + 1


def test_dtime():
    _, _, sys_ = _pendulum()
    ta = hyk.taylor_adaptive(sys=sys_, state=[0.0, 0.25])
    assert ta.dtime == (0.0, 0.0)
    ta.step()
    ta.propagate_for(1001.1)
    assert ta.dtime[1] != 0
    ta.dtime = (1, 0.5)
    assert ta.dtime == (1.5, 0.0)


def test_copy():
    _, v, sys_ = _pendulum()
    ta = hyk.taylor_adaptive(sys=sys_, state=[0.0, 0.25], t_events=[hyk.t_event(v)])
    ta.step()

    class foo:
        pass

    ta.bar = foo()
    assert id(ta.bar) == id(copy(ta).bar)
    assert id(ta.bar) != id(deepcopy(ta).bar)
    assert np.all(ta.state == copy(ta).state)
    assert np.all(ta.state == deepcopy(ta).state)
    ta_dc = deepcopy(ta)
    assert ta_dc.state[0] == ta.state[0]
    ta.state[0] += 1
    assert ta_dc.state[0] != ta.state[0]


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_basic(fp_t):
    _, v, sys_ = _pendulum()
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0.0), fp_t(0.25)], t_events=[hyk.t_event(v, fp_type=fp_t)],
                             fp_type=fp_t)
    assert ta.with_events and not ta.compact_mode and not ta.high_accuracy
    assert ta.sys == sys_
    # without a state, or with an empty one: a zero state
    assert np.all(hyk.taylor_adaptive(sys=sys_, fp_type=fp_t).state == [0, 0])
    assert np.all(hyk.taylor_adaptive(sys=sys_, state=[], fp_type=fp_t).state == [0, 0])
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0.0), fp_t(0.25)], compact_mode=True, high_accuracy=True,
                             fp_type=fp_t)
    assert not ta.with_events and ta.compact_mode and ta.high_accuracy
    assert not ta.llvm_state.fast_math and not ta.llvm_state.force_avx512
    assert ta.llvm_state.opt_level == 3
    # read-only arrays whose writeability cannot be changed
    assert not ta.tc.flags.writeable
    with pytest.raises(ValueError):
        ta.tc.flags.writeable = True
    assert not ta.d_output.flags.writeable
    with pytest.raises(ValueError):
        ta.d_output.flags.writeable = True
    with pytest.warns(UserWarning):
        ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0.0), fp_t(0.25)], compact_mode=True, high_accuracy=True,
                                 force_avx512=True, fast_math=True, opt_level=0, fp_type=fp_t)
    assert ta.llvm_state.fast_math and ta.llvm_state.force_avx512
    assert ta.llvm_state.opt_level == 0

    grid = [fp_t(0.0), fp_t(1.0), fp_t(2.0)]
    cb = _Counter()
    ta.propagate_until(fp_t(10.0), callback=cb)
    assert ta.counter > 0
    orig = ta.counter
    ta.propagate_for(fp_t(10.0), callback=cb)
    assert ta.counter > orig
    orig = ta.counter
    ta.time = fp_t(0.0)
    ta.propagate_grid(grid, callback=cb)
    assert ta.counter > orig

    inst = _SameObject()
    inst.orig_id = id(inst)
    ta.time = fp_t(0.0)
    assert id(ta.propagate_until(fp_t(10.0), callback=inst)[-1]) == id(inst)
    assert id(ta.propagate_for(fp_t(10.0), callback=inst)[-1]) == id(inst)
    ta.time = fp_t(0.0)
    assert id(ta.propagate_grid(grid, callback=inst)[-2]) == id(inst)

    with pytest.raises(TypeError, match="cannot be used as a step callback because it is not callable"):
        ta.time = fp_t(0.0)
        ta.propagate_grid(grid, callback="hello world")
    with pytest.raises(TypeError, match="The call operator of a step callback is expected to return a boolean, "
                                        "but a value of type"):
        ta.time = fp_t(0.0)
        ta.propagate_grid(grid, callback=_Broken())
    for call in (lambda: ta.propagate_until(fp_t(10.0), callback=_Hook()),
                 lambda: ta.propagate_for(fp_t(10.0), callback=_Hook()),
                 lambda: ta.propagate_grid(grid, callback=_Hook())):
        ta.time = fp_t(0.0)
        call()
        assert ta.foo
        delattr(ta, "foo")


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_events(fp_t):
    _, v, sys_ = _pendulum()
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0.0), fp_t(0.25)],
                             nt_events=[hyk.nt_event(v * v - 1e-6, _cb0, fp_type=fp_t)],
                             t_events=[hyk.t_event(v, fp_type=fp_t)], fp_type=fp_t)
    assert ta.with_events and len(ta.t_events) == 1 and len(ta.nt_events) == 1
    oc = ta.propagate_until(fp_t(1e9))[0]
    assert int(oc) == -1
    assert ta.te_cooldowns[0] is not None
    ta.reset_cooldowns()
    assert ta.te_cooldowns[0] is None


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_s11n(fp_t):
    _, v, sys_ = _pendulum()
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0), fp_t(0.25)], fp_type=fp_t,
                             nt_events=[hyk.nt_event(v * v - 1e-10, _cb0, fp_type=fp_t)])
    for _ in range(4):
        ta.step()
    ta2 = pickle.loads(pickle.dumps(ta))
    assert len(ta.t_events) == len(ta2.t_events) and len(ta.nt_events) == len(ta2.nt_events)
    ta.foo = "hello world"
    ta = pickle.loads(pickle.dumps(ta))
    assert ta.foo == "hello world"
    assert np.all(ta.state == ta2.state) and np.all(ta.time == ta2.time)
    ta.step()
    ta2.step()
    assert np.all(ta.state == ta2.state) and np.all(ta.time == ta2.time)

    # a stateful event callback: copied into the event, its state pickled
    clb = _Stateful()
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0), fp_t(0.25)], fp_type=fp_t,
                             nt_events=[hyk.nt_event(v * v - 1e-10, clb, fp_type=fp_t)])
    assert id(clb) != id(ta.nt_events[0].callback)
    assert ta.nt_events[0].callback.n == 0
    ta.propagate_until(fp_t(10))
    ta2 = pickle.loads(pickle.dumps(ta))
    assert ta.nt_events[0].callback.n == ta2.nt_events[0].callback.n
    ta.foo = "hello world"
    ta = pickle.loads(pickle.dumps(ta))
    assert ta.foo == "hello world"
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0), fp_t(0.25)], fp_type=fp_t, tol=fp_t(1e-6))
    assert ta.tol == fp_t(1e-6)


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_step_callback(fp_t):
    x, _, sys_ = _pendulum()
    ta = hyk.taylor_adaptive(sys=sys_, state=[fp_t(0.0), fp_t(10.0)], fp_type=fp_t)
    cb1, cb2 = _Hook(), _Hook()
    res = ta.propagate_for(fp_t(10.0), callback=[cb1, cb2])
    assert isinstance(res[-1], list)
    assert id(res[-1][0]) == id(cb1) and id(res[-1][1]) == id(cb2)
    assert hasattr(ta, "foo")
    res = ta.propagate_until(fp_t(20.0), callback=[cb1, hyk.callback.angle_reducer([x]), cb2])
    assert isinstance(res[-1], list) and isinstance(res[-1][1], hyk.callback.angle_reducer)
    assert id(res[-1][0]) == id(cb1) and id(res[-1][2]) == id(cb2)
    assert fp_t(0) <= ta.state[0] < fp_t(6.29)
    res = ta.propagate_grid([fp_t(20.0), fp_t(30.0)], callback=cb1)
    assert id(res[-2]) == id(cb1)
    res = ta.propagate_for(fp_t(10.0), callback=hyk.callback.angle_reducer([x]))
    assert isinstance(res[-1], hyk.callback.angle_reducer)
    assert fp_t(0) <= ta.state[0] < fp_t(6.29)
