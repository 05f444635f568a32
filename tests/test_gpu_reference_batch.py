"""The reference's batch-integrator tests, restated for the GPU integrator
(heyoka/_test_batch_integrator.py test_copy :89-126, test_propagate_until
:234-338, test_basic :490-553, test_propagate_grid :692-858): the same
systems, initial conditions, calls and checks, in both precisions."""

from copy import copy, deepcopy

import numpy as np
import pytest

import hyk

pytestmark = pytest.mark.gpu

FP_TYPES = [np.float32, float]


def _pendulum():
    x, v = hyk.make_vars("x", "v")
    return x, v, [(x, v), (v, -9.8 * hyk.sin(x))]


def _cb0(ta, t, d_sgn, bidx):
    pass


class _Counter:
    """A step callback that adds a dynamic attribute to the integrator."""

    def __call__(self, ta):
        if hasattr(ta, "counter"):
            ta.counter += 1
        else:
            ta.counter = 0
        return True


class _SameObject:
    """A step callback that checks that it is not copied."""

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


def _check_callbacks(ta, call, reset):
    """The callback checks shared by propagate_until/for/grid."""
    reset()
    call(callback=_Counter())
    assert ta.counter > 0
    inst = _SameObject()
    inst.orig_id = id(inst)
    reset()
    call(callback=inst)
    reset()
    with pytest.raises(TypeError, match="cannot be used as a step callback because it is not callable"):
        call(callback="hello world")
    reset()
    with pytest.raises(TypeError, match="The call operator of a step callback is expected to return a boolean, "
                                        "but a value of type"):
        call(callback=_Broken())
    reset()
    call(callback=_Hook())
    assert ta.foo
    delattr(ta, "foo")


def test_copy():
    x, v, sys_ = _pendulum()
    ta = hyk.taylor_adaptive_batch(sys=sys_, state=[[0, 0.01], [0.25, 0.26]],
                                   nt_events=[hyk.nt_event_batch(v * v - 1e-10, _cb0)])
    for _ in range(4):
        ta.step()

    class foo:
        pass

    ta.bar = foo()
    assert id(ta.bar) == id(copy(ta).bar)
    assert id(ta.bar) != id(deepcopy(ta).bar)
    assert np.all(ta.state == copy(ta).state)
    assert np.all(ta.state == deepcopy(ta).state)
    ta_dc = deepcopy(ta)
    assert ta_dc.state[0, 0] == ta.state[0, 0]
    ta.state[0, 0] += 1
    assert ta_dc.state[0, 0] != ta.state[0, 0]


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_propagate_until(fp_t):
    ic = np.array([[0.0, 0.1, 0.2, 0.3], [0.25, 0.26, 0.27, 0.28]], dtype=fp_t)
    _, _, sys_ = _pendulum()
    ta = hyk.taylor_adaptive_batch(sys=sys_, state=ic, fp_type=fp_t)

    def reset():
        ta.set_time(fp_t(0.0))
        ta.state[:] = ic

    # vector and scalar end times and max_delta_t give the same bits
    ta.propagate_until([fp_t(10.0)] * 4)
    st, res = deepcopy(np.asarray(ta.state)), deepcopy(ta.propagate_res)
    reset()
    ta.propagate_until(fp_t(10.0))
    assert np.all(ta.state == st) and res == ta.propagate_res
    reset()
    ta.propagate_until([fp_t(10.0)] * 4, max_delta_t=[fp_t(1e-4)] * 4)
    st, res = deepcopy(np.asarray(ta.state)), deepcopy(ta.propagate_res)
    reset()
    ta.propagate_until(fp_t(10.0), max_delta_t=fp_t(1e-4))
    assert np.all(ta.state == st) and res == ta.propagate_res
    _check_callbacks(ta, lambda **kw: ta.propagate_until(fp_t(10.0), **kw), reset)


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_basic(fp_t):
    x, v, sys_ = _pendulum()
    st = np.array([[0.0, 0.1], [0.25, 0.26]], dtype=fp_t)
    ta = hyk.taylor_adaptive_batch(sys=sys_, state=st, t_events=[hyk.t_event_batch(v, fp_type=fp_t)], fp_type=fp_t)
    assert ta.with_events and not ta.compact_mode and not ta.high_accuracy
    assert ta.sys == sys_
    ta = hyk.taylor_adaptive_batch(sys=sys_, state=st, compact_mode=True, high_accuracy=True, fp_type=fp_t)
    assert not ta.with_events and ta.compact_mode and ta.high_accuracy
    assert not ta.llvm_state.fast_math and not ta.llvm_state.force_avx512
    assert ta.llvm_state.opt_level == 3
    # an empty initial state: a zero state of batch size 2
    ta = hyk.taylor_adaptive_batch(sys=sys_, state=np.empty((0, 2), dtype=fp_t), compact_mode=True,
                                   high_accuracy=True, fp_type=fp_t)
    assert np.all(ta.state == np.zeros((2, 2), dtype=fp_t))
    with pytest.warns(UserWarning):
        ta = hyk.taylor_adaptive_batch(sys=sys_, state=st, compact_mode=True, high_accuracy=True,
                                       force_avx512=True, fast_math=True, opt_level=0, fp_type=fp_t)
    assert ta.llvm_state.fast_math and ta.llvm_state.force_avx512
    assert ta.llvm_state.opt_level == 0


@pytest.mark.parametrize("fp_t", FP_TYPES)
def test_propagate_grid(fp_t):
    _, _, sys_ = _pendulum()
    x_ic = np.array([0.06, 0.07, 0.08, 0.09], dtype=fp_t)
    v_ic = np.array([0.025, 0.026, 0.027, 0.028], dtype=fp_t)
    ta = hyk.taylor_adaptive_batch(sys_, [x_ic, v_ic], fp_type=fp_t)

    with pytest.raises(ValueError, match=r"Invalid grid passed to the propagate_grid\(\) method of a batch "
                                         r"integrator: the expected number of dimensions is 2, but the input "
                                         r"array has a dimension of 1"):
        ta.propagate_grid(np.array([], dtype=fp_t))
    with pytest.raises(ValueError, match=r"Invalid grid passed to the propagate_grid\(\) method of a batch "
                                         r"integrator: the shape must be \(n, 4\) but the number of columns "
                                         r"is 2 instead"):
        ta.propagate_grid(np.array([[1, 2], [3, 4]], dtype=fp_t))

    # batch against four scalar integrators
    tas = [hyk.taylor_adaptive(sys_, [x0, v0], fp_type=fp_t) for x0, v0 in zip(x_ic, v_ic)]
    grid = np.array([[-0.1, -0.2, -0.3, -0.4], [0.01, 0.02, 0.03, 0.9], [1.0, 1.1, 1.2, 1.3],
                     [11.0, 11.1, 11.2, 11.3]], dtype=fp_t)
    ta.propagate_until(grid[0, :])
    bres = ta.propagate_grid(grid)
    assert bres[0] is None
    for idx, cur in enumerate(tas):
        cur.propagate_until(grid[0, idx])
    sres = [cur.propagate_grid(grid[:, idx]) for idx, cur in enumerate(tas)]
    for idx in range(4):
        assert np.max(np.abs(sres[idx][5] - bres[1][:, :, idx]).flatten()) < np.finfo(fp_t).eps * 100

    def reset():
        ta.set_time(fp_t(0.0))
        ta.state[:] = [x_ic, v_ic]
        ta.propagate_until(grid[0, :])

    # vector and scalar max_delta_t give the same bits
    reset()
    bres = ta.propagate_grid(grid, max_delta_t=[fp_t(1e-3)] * 4)
    res = deepcopy(ta.propagate_res)
    reset()
    bres2 = ta.propagate_grid(grid, max_delta_t=fp_t(1e-3))
    assert np.all(bres[1] == bres2[1])
    assert ta.propagate_res == res
    _check_callbacks(ta, lambda **kw: ta.propagate_grid(grid, **kw), reset)
