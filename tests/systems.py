"""ODE systems shared by several tests: together they cover every operation
and operand kind of the code generator (variables, numbers, parameters, the
time; add, sub, mul, div, neg, square, sqrt, pow, exp, log, sin, cos) and
time-constant operations, beyond what the benchmark systems use."""

import numpy as np

import hyk


def mixed():
    x, y = hyk.make_vars("x", "y")
    t, p = hyk.time, hyk.par
    return [
        (x, hyk.exp(-y) * hyk.log(x) + hyk.sqrt(y) / x + hyk.cos(t) * p[1] + p[0] / y + x * t + 0.5 * t),
        (y, p[0] / (x + 2.0) - x**-1.5 * p[1] + hyk.sin(x) * y + hyk.square(x - y) + t * y - (3.0 - x)
         + hyk.exp(t) * 1e-3 + y**2.5 + (x - t) / 7.0 + 2.0 - t),
    ]


def consts():
    # time-constant operations (only an order-0 value) feeding every kind of operation
    x, y = hyk.make_vars("x", "y")
    p = hyk.par
    c1, c2 = 1.0 - p[0], hyk.exp(p[1])
    return [
        (x, c1 * y + c2 * hyk.sin(x) + hyk.sqrt(p[0] + 2.0) - (p[0] * 3.0) / (x + 4.0) + y / (p[1] + 1.0)),
        (y, -x * hyk.sin(p[1]) + hyk.cos(p[0] * x) + (c1 - y) ** 2.0 + hyk.log(c2 + x * x) - c1),
    ]


def var2():
    """Order-2 variational equations of the forced damped pendulum (with
    respect to the initial state and the parameter)."""
    from hyk import var

    x, v = hyk.make_vars("x", "v")
    orig = [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]
    return var.var_ode_sys(orig, var.var_args.vars | var.var_args.params, order=2)


def var2_state(n, rng):
    """Initial state of var2() for n lanes: pendulum states near (0.2, 0.3)
    and the identity variational state."""
    vs = var2()
    base = np.array([[0.2], [0.3]]) + 0.01 * rng.standard_normal((2, n))
    return np.concatenate([base, vs.initial_variational_state(n)])
