"""First-order variational equations (heyoka/_test_var_integrator.py:144-201
layout) and their sensitivities against central finite differences."""

import numpy as np
import pytest

import hyk
from hyk import var


def forced():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]


def test_layout():
    vs = var.var_ode_sys(forced(), var.var_args.vars)
    assert vs.vslice(0) == slice(0, 2) and vs.vslice(0, 1) == slice(1, 2)
    assert vs.vslice(1) == slice(2, 6) and vs.vslice(1, 1) == slice(4, 6)
    assert [vs.mindex(i) for i in range(6)] == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1]]
    x, v = hyk.make_vars("x", "v")
    assert vs.vargs == [x, v]
    vs = var.var_ode_sys(forced(), var.var_args.all & ~var.var_args.time)
    assert len(vs.vargs) == 3 and len(vs.sys) == 2 + 2 * 3


def test_diff_rules():
    x, y = hyk.make_vars("x", "y")
    e = hyk.sin(x) * y**-1.5 + hyk.exp(x / y) - hyk.log(hyk.sqrt(x))
    for var_, h in ((x, 1e-6), (y, 1e-6)):
        d = hyk.diff(e, var_)
        import math

        def ev(ex, xv, yv):
            from hyk import expr as E

            def f(n):
                if n.kind == E.VAR:
                    return {"x": xv, "y": yv}[n.value]
                if n.kind == E.NUM:
                    return n.value
                a = [f(c) for c in n.args]
                fn = n.value
                return {
                    "add": lambda: a[0] + a[1], "sub": lambda: a[0] - a[1], "mul": lambda: a[0] * a[1],
                    "div": lambda: a[0] / a[1], "neg": lambda: -a[0], "square": lambda: a[0] * a[0],
                    "sqrt": lambda: math.sqrt(a[0]), "pow": lambda: a[0] ** a[1], "exp": lambda: math.exp(a[0]),
                    "log": lambda: math.log(a[0]), "sin": lambda: math.sin(a[0]), "cos": lambda: math.cos(a[0]),
                }[fn]()

            return f(ex)

        x0, y0 = 0.7, 1.3
        if var_ is x:
            fd = (ev(e, x0 + h, y0) - ev(e, x0 - h, y0)) / (2 * h)
        else:
            fd = (ev(e, x0, y0 + h) - ev(e, x0, y0 - h)) / (2 * h)
        assert abs(ev(d, x0, y0) - fd) < 1e-8


def test_sensitivities_vs_finite_differences(oracle):
    vs = var.var_ode_sys(forced(), var.var_args.vars | var.var_args.params)
    st0 = np.array([[0.2, 0.21], [0.3, 0.31]])
    pars = np.array([[0.4, 0.41]])
    full = np.concatenate([st0, vs.initial_variational_state(2)])
    o = oracle.Oracle(vs.sys, full, pars=pars, order=20, mode=1)
    o.propagate_until(3.0)
    sens = o.state[2:].reshape(2, 3, 2)  # [component][arg][lane]
    eps = 1e-6
    for j in range(3):
        plus, minus = st0.copy(), st0.copy()
        pp, pm = pars.copy(), pars.copy()
        if j < 2:
            plus[j] += eps
            minus[j] -= eps
        else:
            pp[0] += eps
            pm[0] -= eps
        a = oracle.Oracle(forced(), plus, pars=pp, order=20, mode=1)
        b = oracle.Oracle(forced(), minus, pars=pm, order=20, mode=1)
        a.propagate_until(3.0)
        b.propagate_until(3.0)
        fd = (a.state - b.state) / (2 * eps)
        assert np.max(np.abs(fd - sens[:, j, :])) < 1e-7
