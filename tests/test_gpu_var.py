"""The batch variational API on the GPU (heyoka/_test_var_integrator.py:144-258):
an order-2 variational system, its properties, ``tstate`` and
``eval_taylor_map``, and bit-for-bit parity of the augmented state with the
oracle."""

from sys import getrefcount

import numpy as np
import pytest

import hyk
from hyk import var

pytestmark = pytest.mark.gpu


def forced():
    x, v = hyk.make_vars("x", "v")
    return x, v, [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]


def test_reference_batch_variational(oracle):
    x, v, orig = forced()
    vsys = var.var_ode_sys(orig, var.var_args.vars, order=2)
    ta = hyk.taylor_adaptive_batch(vsys, [[0.2, 0.21], [0.3, 0.31]], pars=[[0.4, 0.41]], time=[0.5, 0.51],
                                   compact_mode=True)
    assert ta.dim > 2 and ta.n_orig_sv == 2 and ta.is_variational and ta.vorder == 2 and ta.vargs == [x, v]
    rc = getrefcount(ta)
    ts = ta.tstate
    assert ts.shape == (2, 2) and np.all(ts == 0.0)
    with pytest.raises(ValueError):
        ta.tstate[0] = 0.5
    assert ta.get_vslice(order=1) == slice(2, 6) and ta.get_vslice(order=1, component=1) == slice(4, 6)
    assert ta.get_mindex(4) == [1, 1, 0] and ta.get_mindex(i=5) == [1, 0, 1]
    ta.propagate_until(3.0)
    ts2 = ta.eval_taylor_map([[0.0, 0.0], [0.0, 0.0]])
    assert np.shares_memory(ts, ts2)
    assert np.all(ts2 == np.asarray(ta.state)[:2])
    ts2 = ta.eval_taylor_map(np.array([[0.0, 0.0], [0.0, 0.0]]))
    assert np.all(ts2 == np.asarray(ta.state)[:2])
    with pytest.raises(TypeError, match="Invalid dtype detected for the inputs of a Taylor map evaluation:"):
        ta.eval_taylor_map(np.array([[0, 0], [0, 0]], dtype=np.int32))
    with pytest.raises(ValueError, match="the array is not C-style contiguous, please "):
        ta.eval_taylor_map(np.zeros((2, 4))[:, ::2])
    with pytest.raises(ValueError, match="has 1 dimension"):
        ta.eval_taylor_map(np.array([0.0, 0.0]))
    with pytest.raises(ValueError, match="has 1 row\\(s\\), but it must have 2 row\\(s\\) instead"):
        ta.eval_taylor_map(np.array([[0.0, 0.0]]))
    with pytest.raises(ValueError, match="has 1 column\\(s\\), but it must have 2 column\\(s\\) instead"):
        ta.eval_taylor_map(np.array([[0.0], [0.0]]))
    with pytest.raises(ValueError, match="may overlap"):
        ta.eval_taylor_map(ta.state[:2])
    with pytest.raises(ValueError, match="may overlap"):
        ta.eval_taylor_map(ta.tstate)
    # the augmented state equals the oracle's, bit for bit
    full = np.concatenate([np.array([[0.2, 0.21], [0.3, 0.31]]), vsys.initial_variational_state(2)])
    o = oracle.Oracle(vsys.sys, full, pars=[[0.4, 0.41]], time=[0.5, 0.51], order=ta.order, mode=1)
    o.propagate_until(3.0)
    assert np.array_equal(np.asarray(ta.state), o.state)


def test_taylor_map_predicts_perturbed_flow():
    x, v, orig = forced()
    vsys = var.var_ode_sys(orig, var.var_args.vars | var.var_args.params, order=2)
    st = np.array([[0.2, 0.25, 0.3], [0.3, 0.2, 0.1]])
    ta = hyk.taylor_adaptive_batch(vsys, st, pars=[[0.4, 0.4, 0.4]])
    ta.propagate_until(2.0)
    d = np.array([[1e-3, -2e-3, 0.0], [0.0, 1e-3, -1e-3], [5e-4, 0.0, 1e-3]])
    pred = ta.eval_taylor_map(d).copy()
    ref = hyk.taylor_adaptive_batch(orig, st + d[:2], pars=[[0.4, 0.4, 0.4]] + d[2:3])
    ref.propagate_until(2.0)
    err = np.max(np.abs(pred - np.asarray(ref.state)))
    assert err < 1e-7  # third-order remainder of displacements ~1e-3


def test_initial_time_variational_integrator_bitwise(oracle):
    """A variational integrator with the initial time among its arguments:
    the constructor fills the t0 derivatives' initial values from the state,
    the parameters and the initial times; the propagation matches the oracle
    bit for bit."""
    x, v = hyk.make_vars("x", "v")
    orig = [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]
    vs = hyk.var_ode_sys(orig, [v, hyk.time, x], order=2)
    x0 = np.array([[0.2, -0.4, 0.1], [0.3, 0.1, -0.2]])
    pars = np.array([[0.4, 0.25, 0.1]])
    t0 = np.array([0.5, 0.6, -0.2])
    ta = hyk.taylor_adaptive_batch(vs, x0, pars=pars, time=t0)
    full0 = np.asarray(ta.state).copy()
    assert np.array_equal(full0[2:], vs.initial_variational_state_at(x0, t0, pars))
    ta.propagate_until(3.0)
    o = oracle.Oracle(vs.sys, full0, pars=pars, time=t0, order=ta.order, mode=1)
    o.propagate_until(3.0)
    assert np.array_equal(np.asarray(ta.state), o.state)


def test_reference_scalar_variational_integrator():
    """heyoka/_test_var_integrator.py test_scalar (:14-110): a scalar
    integrator of a second-order variational system, tstate that keeps the
    integrator alive, the variable ordering, eval_taylor_map and its errors."""
    x, v = hyk.make_vars("x", "v")
    orig_sys = [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]
    vsys = hyk.var_ode_sys(orig_sys, hyk.var_args.vars, order=2)
    ta = hyk.taylor_adaptive(vsys, [0.2, 0.3], pars=[0.4], time=0.5, compact_mode=True)
    assert ta.dim > 2 and ta.n_orig_sv == 2 and ta.is_variational
    assert ta.vorder == 2 and ta.vargs == [x, v]
    rc = getrefcount(ta)
    ts = ta.tstate
    assert getrefcount(ta) == rc + 1
    assert ts.shape == (2,) and np.all(ts == [0.0, 0.0])
    with pytest.raises(ValueError):
        ta.tstate[0] = 0.5
    assert ta.get_vslice(order=0) == slice(0, 2, None)
    assert ta.get_vslice(order=0, component=1) == slice(1, 2, None)
    assert ta.get_vslice(order=1) == slice(2, 6, None)
    assert ta.get_vslice(order=1, component=1) == slice(4, 6, None)
    assert ta.get_mindex(0) == [0, 0, 0] and ta.get_mindex(1) == [1, 0, 0]
    assert ta.get_mindex(2) == [0, 1, 0] and ta.get_mindex(3) == [0, 0, 1]
    assert ta.get_mindex(4) == [1, 1, 0] and ta.get_mindex(i=5) == [1, 0, 1]
    ta.propagate_until(3.0)
    ts2 = ta.eval_taylor_map([0.0, 0.0])
    assert getrefcount(ta) == rc + 2
    assert np.shares_memory(ts, ts2) and np.all(ts2 == np.asarray(ta.state[:2].cpu()))
    ts2 = ta.eval_taylor_map(np.array([0.0, 0.0]))
    assert np.shares_memory(ts, ts2) and np.all(ts2 == np.asarray(ta.state[:2].cpu()))
    with pytest.raises(TypeError, match="Invalid dtype detected for the inputs of a Taylor map evaluation:"):
        ta.eval_taylor_map(np.array([0.0, 0.0], dtype=np.int32))
    with pytest.raises(ValueError, match="Invalid inputs array detected in a Taylor map evaluation: the array is not "
                                         "C-style contiguous, please "):
        ta.eval_taylor_map(np.array([0.0, 0.0, 0.0, 0.0])[::2])
    with pytest.raises(ValueError, match="The array of inputs provided for the evaluation of a Taylor map has 2 "
                                         "dimensions, "):
        ta.eval_taylor_map(np.array([[0.0, 0.0], [0.0, 0.0]]))
    with pytest.raises(ValueError, match="The array of inputs provided for the evaluation of a Taylor map has 4 "
                                         "elements, "):
        ta.eval_taylor_map(np.array([0.0, 0.0, 0.0, 0.0]))
    with pytest.raises(ValueError, match="may overlap"):
        ta.eval_taylor_map(ta.state[:2])
    with pytest.raises(ValueError, match="may overlap"):
        ta.eval_taylor_map(ta.tstate)


def test_reference_taylor_map_size_check():
    """heyoka/_test_var_integrator.py test_size_check_bug: the inputs of a
    Taylor map are sized by the variational arguments (here 3: x, v and the
    parameter), not by the original state variables."""
    x, v = hyk.make_vars("x", "v")
    orig_sys = [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]
    vsys = hyk.var_ode_sys(orig_sys, hyk.var_args.vars | hyk.var_args.params, order=2)
    ta = hyk.taylor_adaptive(vsys, [0.2, 0.3], pars=[0.4], time=0.5, compact_mode=True)
    assert np.all(ta.state[:2] == ta.eval_taylor_map([0.0, 0.0, 0.0]))
    ta = hyk.taylor_adaptive_batch(vsys, [[0.2, 0.21], [0.3, 0.31]], pars=[[0.4, 0.41]], time=[0.5, 0.51],
                                   compact_mode=True)
    assert np.all(ta.state[:2] == ta.eval_taylor_map([[0.0, 0.0], [0.0, 0.0], [0.0, 0.0]]))
