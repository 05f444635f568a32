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


def test_order2_layout():
    vs = var.var_ode_sys(forced(), var.var_args.vars, order=2)
    # the reference's pinned part (heyoka/_test_var_integrator.py:54-65)
    assert vs.vslice(0) == slice(0, 2) and vs.vslice(1) == slice(2, 6) and vs.vslice(1, 1) == slice(4, 6)
    assert [vs.mindex(i) for i in range(6)] == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1]]
    # order 2: per component the multi-indices (2,0), (1,1), (0,2)
    assert vs.vslice(2) == slice(6, 12) and vs.vslice(2, 1) == slice(9, 12)
    assert [vs.mindex(i) for i in range(6, 12)] == [[0, 2, 0], [0, 1, 1], [0, 0, 2], [1, 2, 0], [1, 1, 1], [1, 0, 2]]
    assert len(vs.sys) == 12 and vs.order == 2
    init = vs.initial_variational_state(3)
    assert init.shape == (10, 3) and np.array_equal(init[:4, 0], [1.0, 0.0, 0.0, 1.0]) and not init[4:].any()


def test_order2_sensitivities_vs_finite_differences(oracle):
    """Second derivatives of the flow (state and parameter arguments) against
    central differences of the first-order sensitivities."""
    vs2 = var.var_ode_sys(forced(), var.var_args.vars | var.var_args.params, order=2)
    vs1 = var.var_ode_sys(forced(), var.var_args.vars | var.var_args.params, order=1)
    st0 = np.array([[0.2, 0.21], [0.3, 0.31]])
    pars = np.array([[0.4, 0.41]])
    o = oracle.Oracle(vs2.sys, np.concatenate([st0, vs2.initial_variational_state(2)]), pars=pars, order=20, mode=1)
    o.propagate_until(3.0)
    m = 3
    mi2 = [vs2.mindex(i) for i in range(vs2.vslice(2).start, vs2.vslice(2).stop)]
    eps = 1e-5
    for j in range(m):
        plus, minus = st0.copy(), st0.copy()
        pp, pm = pars.copy(), pars.copy()
        if j < 2:
            plus[j] += eps
            minus[j] -= eps
        else:
            pp[0] += eps
            pm[0] -= eps
        a = oracle.Oracle(vs1.sys, np.concatenate([plus, vs1.initial_variational_state(2)]), pars=pp, order=20, mode=1)
        b = oracle.Oracle(vs1.sys, np.concatenate([minus, vs1.initial_variational_state(2)]), pars=pm, order=20,
                          mode=1)
        a.propagate_until(3.0)
        b.propagate_until(3.0)
        d1 = (a.state[2:] - b.state[2:]).reshape(2, m, 2) / (2 * eps)  # d/da_j of dx_i/da_k
        for row, mi in zip(range(vs2.vslice(2).start, vs2.vslice(2).stop), mi2):
            comp, alpha = mi[0], mi[1:]
            if alpha[j] == 0:
                continue
            k = [q for q in range(m) if alpha[q] - (1 if q == j else 0) > 0][0]
            assert np.max(np.abs(o.state[row] - d1[comp, k])) < 1e-6, (row, mi, j)


def _fd_t0(oracle, sys_, x0, pars, t0, t1, d):
    """x(t1) for initial times t0 - d, t0, t0 + d (same x0), on the oracle."""
    out = []
    for s in (-d, 0.0, d):
        o = oracle.Oracle(sys_, x0, pars=pars, time=np.full(x0.shape[1], t0 + s), order=20, mode=1)
        o.propagate_until(t1)
        out.append(o.state.copy())
    return out


def test_initial_time_sensitivities_vs_finite_differences(oracle):
    """Derivatives with respect to the initial time (non-autonomous forced
    pendulum): order 1 and 2 in t0 and the mixed t0 / x0 derivative, against
    central differences of integrations started at shifted times."""
    x, v = hyk.make_vars("x", "v")
    orig = forced()
    vs = var.var_ode_sys(orig, [v, hyk.time, x], order=2)
    assert vs.vargs == [v, hyk.time, x] and vs.has_time
    x0 = np.array([[0.2, -0.4], [0.3, 0.1]])
    pars = np.array([[0.4, 0.25]])
    t0, t1 = 0.5, 3.0
    ic = vs.initial_variational_state_at(x0, t0, pars)
    o = oracle.Oracle(vs.sys, np.concatenate([x0, ic]), pars=pars, time=np.full(2, t0), order=20, mode=1)
    o.propagate_until(t1)
    full = o.state
    # order 1 in t0: component i, multi-index (0, 1, 0)
    sl1 = vs.vslice(1)
    m1 = vs._mi[1]
    j_t = m1.index([0, 1, 0])
    d1 = 1e-5
    a, c, b = _fd_t0(oracle, orig, x0, pars, t0, t1, d1)
    fd1 = (b - a) / (2 * d1)
    for i in range(2):
        got = full[sl1.start + i * len(m1) + j_t]
        assert np.allclose(got, fd1[i], rtol=1e-7, atol=1e-9), (i, got, fd1[i])
    # order 2 in t0: multi-index (0, 2, 0)
    sl2 = vs.vslice(2)
    m2 = vs._mi[2]
    j_tt = m2.index([0, 2, 0])
    d2 = 1e-3
    a, c, b = _fd_t0(oracle, orig, x0, pars, t0, t1, d2)
    fd2 = (b - 2 * c + a) / d2**2
    for i in range(2):
        got = full[sl2.start + i * len(m2) + j_tt]
        assert np.allclose(got, fd2[i], rtol=1e-4, atol=1e-6), (i, got, fd2[i])
    # mixed t0 / x0: multi-index (0, 1, 1) = d^2 x / dt0 dx0, from central
    # differences in x0 of the order-1 t0 derivative
    vs1 = var.var_ode_sys(orig, [hyk.time], order=1)
    d3 = 1e-5
    vals = []
    for s in (-d3, d3):
        xs = x0.copy()
        xs[0] += s
        ic1 = vs1.initial_variational_state_at(xs, t0, pars)
        oo = oracle.Oracle(vs1.sys, np.concatenate([xs, ic1]), pars=pars, time=np.full(2, t0), order=20, mode=1)
        oo.propagate_until(t1)
        vals.append(oo.state[2:4].copy())
    fd3 = (vals[1] - vals[0]) / (2 * d3)
    j_tx = m2.index([0, 1, 1])
    for i in range(2):
        got = full[sl2.start + i * len(m2) + j_tx]
        assert np.allclose(got, fd3[i], rtol=1e-6, atol=1e-8), (i, got, fd3[i])


def test_var_args_time_order_and_errors():
    x, v = hyk.make_vars("x", "v")
    vs = var.var_ode_sys(forced(), var.var_args.all)
    assert vs.vargs == [x, v, hyk.par[0], hyk.time]
    assert var.var_args.vars | var.var_args.time | var.var_args.params == var.var_args.all
    with pytest.raises(ValueError, match="variational arguments"):
        var.var_ode_sys(forced(), [hyk.sin(x)])
