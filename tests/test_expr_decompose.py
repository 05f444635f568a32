"""Expression system, Taylor decomposition and model factories (CPU only)."""

import math

import pytest

import hyk
from hyk import decompose as D
from hyk import model


def test_folding():
    x, v = hyk.make_vars("x", "v")
    assert (x * 0.0) == hyk.expression(0.0)
    assert (x * 1.0) == x and (x + 0.0) == x and (0.0 + x) == x
    assert -(-x) == x
    assert hyk.expression(2.0) * 3.0 == hyk.expression(6.0)
    assert x**1.0 == x and x**0.0 == hyk.expression(1.0)
    assert hyk.sin(hyk.expression(0.5)) == hyk.expression(math.sin(0.5))
    assert hash(x + v) == hash(hyk.make_vars("x") + hyk.make_vars("v"))


def test_make_vars_errors():
    with pytest.raises(ValueError):
        hyk.make_vars()


def test_pendulum_decomposition():
    x, v = hyk.make_vars("x", "v")
    d = D.taylor_decompose([(x, v), (v, -9.8 * hyk.sin(x))])
    assert d.n_eq == 2 and d.n_pars == 0
    ops = [D.OP_NAMES[o[0]] for o in d.ops]
    assert ops == ["sin", "cos", "mul"]
    # sin/cos are a coupled pair
    assert d.ops[0][1] == 3 and d.ops[1][1] == 2
    # rhs: x' = u_1 (v), v' = u_4
    assert d.rhs[0] == (D.ARG_U, 1, 0.0) and d.rhs[1] == (D.ARG_U, 4, 0.0)
    lst = d.as_list()
    assert len(lst) == 2 + 3 + 2


def test_cse_and_params():
    x, y = hyk.make_vars("x", "y")
    r = (x**2 + y**2) ** -1.5
    d = D.taylor_decompose([(x, y * r), (y, -x * r + hyk.par[2])])
    names = [D.OP_NAMES[o[0]] for o in d.ops]
    assert names.count("pow") == 1 and names.count("square") == 2
    assert d.n_pars == 3


def test_decompose_errors():
    x, v = hyk.make_vars("x", "v")
    with pytest.raises(ValueError, match="not a state variable"):
        D.taylor_decompose([(x, v)])
    with pytest.raises(ValueError, match="twice"):
        D.taylor_decompose([(x, x), (x, x)])
    with pytest.raises(ValueError):
        D.taylor_decompose([])


def test_digest_stable():
    s1 = hyk.workloads.kepler_sys() if hasattr(hyk, "workloads") else None
    from hyk import workloads as W

    assert D.taylor_decompose(W.kepler_sys()).digest() == D.taylor_decompose(W.kepler_sys()).digest()
    assert D.taylor_decompose(W.kepler_sys()).digest() != D.taylor_decompose(W.pendulum_sys()).digest()
    del s1


def test_models():
    x, v = hyk.make_vars("x", "v")
    dyn = model.pendulum()
    assert dyn[0] == (x, v) and dyn[1][1] == -hyk.sin(x)
    assert model.pendulum(gconst=2.0)[1][1] == -2.0 * hyk.sin(x)
    assert model.pendulum(gconst=4.0, length=2.0)[1][1] == -2.0 * hyk.sin(x)
    dyn = model.nbody(2, masses=[0.0, 0.0])
    assert len(dyn) == 12
    for k in (3, 4, 5, 9, 10, 11):
        assert dyn[k][1] == hyk.expression(0.0)
    assert [str(p[0]) for p in dyn[:6]] == ["x_0", "y_0", "z_0", "vx_0", "vy_0", "vz_0"]
    dyn = model.cr3bp()
    xx, px, y = hyk.make_vars("x", "px", "y")
    assert dyn[0][0] == xx and dyn[0][1] == px + y
    assert len(D.taylor_decompose(model.nbody(6)).ops) > 100


def test_default_constructed_continuous_outputs():
    """heyoka/test.py c_output_test_case: default-constructed continuous
    outputs (no device needed)."""
    import pickle
    from copy import copy, deepcopy

    import numpy as np

    import hyk

    for c in (hyk.continuous_output_batch_dbl(), hyk.continuous_output_batch_flt()):
        for obj in (c, copy(c), deepcopy(c), pickle.loads(pickle.dumps(c))):
            with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output_batch object"):
                obj(np.zeros((0,)))
            with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output_batch object"):
                obj(time=[0.0, 0.0])
            assert obj.output is None and obj.times is None and obj.tcs is None
            with pytest.raises(ValueError, match="default-constructed"):
                obj.bounds
            with pytest.raises(ValueError, match="default-constructed"):
                obj.n_steps
            assert obj.batch_size == 0 and "forward" not in repr(obj) and obj.llvm_state.ir != ""
    s = hyk.continuous_output()
    with pytest.raises(ValueError, match="Cannot use a default-constructed continuous_output object"):
        s(1.0)
    assert s.times is None and s.tcs is None and "forward" not in repr(s)
