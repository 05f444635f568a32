"""Variational equations: ``var_ode_sys(sys, args, order)``.

Restates the reference's variational ODE construction
(heyoka/expose_var_ode_sys.cpp:29-59, batch variational API
heyoka/expose_batch_integrators.cpp:549-649): the system is augmented with
the partial derivatives of every state variable with respect to the chosen
arguments (initial values of state variables and/or runtime parameters) up to
the given order.  With X_{i,alpha} = d^|alpha| x_i / d a^alpha for a
multi-index alpha over the m arguments,

    d/dt X_{i,e_j} = D_j f_i,   d/dt X_{i,alpha} = D_k (d/dt X_{i,alpha - e_k}),

where k is the last argument with alpha_k > 0 and D_k is the total
derivative along argument k: D_k g = sum over the variables v of g of
(dg/dv) (dv/da_k) + dg/da_k (a_k a parameter), with dx_l/da_k = X_{l,e_k} and
dX_{l,beta}/da_k = X_{l,beta + e_k}.

The initial time t0 is an argument like an initial condition (the right-hand
side depends on t0 only through the state), with initial values from the
flow's time-shift structure: x(t; t0, x0) = Psi(t - t0; x0, s0 = t0) for the
flow Psi of the system made autonomous by the state s' = 1, so
d/dt0 = -d/dtau + d/ds0 and, at t = t0, for k >= 1 derivatives in t0,
beta in the state arguments and gamma in the parameters,

    X_{i,alpha}(t0) = sum_{j=1..k} C(k, j) (-1)^j d_t^(k-j) d_x^beta d_p^gamma L^j(x_i),

with L g = sum_l f_l dg/dx_l + dg/dt the Lie derivative along the system
(L^j(x_i) / j! is the order-j Taylor coefficient of x_i), evaluated at
(x0, t0, p).

Layout (heyoka/_test_var_integrator.py:54-65 pins it up to order 1): the
original state, then for each order 1, 2, ... and each component i, the
multi-indices of that order in decreasing lexicographic order ((1,0) before
(0,1); (2,0), (1,1), (0,2) at order 2).  Initial values: the identity for
state arguments at order 1, zero otherwise.
"""

from __future__ import annotations

import enum
import math

from . import expr as _e


class var_args(enum.IntFlag):
    vars = 1
    params = 2
    time = 4
    all = 7


def _multi_indices(m, r):
    """The multi-indices of total order r over m arguments, decreasing lexicographic."""
    out = []

    def rec(prefix, left, k):
        if k == m - 1:
            out.append(prefix + [left])
            return
        for a in range(left, -1, -1):
            rec(prefix + [a], left - a, k + 1)

    if m == 0:
        return [] if r else [[]]
    rec([], r, 0)
    return out


class var_ode_sys:
    def __init__(self, sys, args=var_args.vars, order=1):
        order = int(order)
        if order < 1:
            raise ValueError("The order of a variational ODE system must be at least 1")
        pairs = [(_e._ex(l), _e._ex(r)) for l, r in sys]
        xs = [l for l, _ in pairs]
        if isinstance(args, var_args):
            vargs = []
            if args & var_args.vars:
                vargs += xs
            if args & var_args.params:
                npar = 0
                stack = [r for _, r in pairs]
                while stack:
                    n = stack.pop()
                    if n.kind == _e.PAR:
                        npar = max(npar, n.value + 1)
                    stack.extend(n.args)
                vargs += [_e.par[i] for i in range(npar)]
            if args & var_args.time:
                vargs.append(_e.time)
        else:
            vargs = [_e._ex(a) for a in args]
            for a in vargs:
                if not (a.kind in (_e.PAR, _e.TIME) or (a.kind == _e.VAR and a in xs)):
                    raise ValueError("variational arguments must be state variables, parameters or the time")
        n, m = len(pairs), len(vargs)
        self.n_orig_sv = n
        self._orig = pairs
        self.vargs = vargs
        self.order = order
        # multi-indices per order, and the variable of each (component, multi-index)
        self._mi = {r: _multi_indices(m, r) for r in range(1, order + 1)}
        var_of = {}
        for r in range(1, order + 1):
            for i in range(n):
                for a in self._mi[r]:
                    var_of[(i, tuple(a))] = _e.make_vars("d_{}_{}".format(i, "_".join(map(str, a))))
        self._var_of = var_of
        # d(variable)/d(a_k) for the variables of the augmented state
        xidx = {x.value: i for i, x in enumerate(xs)}
        vidx = {v.value: key for key, v in var_of.items()}

        def dvar(v, k):
            e = [0] * m
            e[k] = 1
            if v.value in xidx:
                return var_of[(xidx[v.value], tuple(e))]
            i, a = vidx[v.value]
            b = tuple(x + y for x, y in zip(a, e))
            return var_of.get((i, b))  # None beyond the order (never needed)

        def total(g, k):
            terms = []
            for name in _e.get_variables(g):
                v = _e.expression(name)
                dg = _e.diff(g, v)
                if dg.kind == _e.NUM and dg.value == 0.0:
                    continue
                terms.append(dg * dvar(v, k))
            a = vargs[k]
            if a.kind == _e.PAR:
                terms.append(_e.diff(g, a))
            return _e.sum(terms)

        rhs = {}
        out = list(pairs)
        for r in range(1, order + 1):
            for i in range(n):
                for a in self._mi[r]:
                    k = max(j for j in range(m) if a[j] > 0)
                    if r == 1:
                        g = total(pairs[i][1], k)
                    else:
                        b = list(a)
                        b[k] -= 1
                        g = total(rhs[(i, tuple(b))], k)
                    rhs[(i, tuple(a))] = g
                    out.append((var_of[(i, tuple(a))], g))
        self.sys = out

    def initial_variational_state(self, B):
        """The initial values of the derivatives, shape (n_derivatives, B)."""
        import numpy as np

        n, m = self.n_orig_sv, len(self.vargs)
        rows = []
        for r in range(1, self.order + 1):
            for i in range(n):
                for a in self._mi[r]:
                    one = r == 1 and self.vargs[a.index(1)].kind == _e.VAR and self.vargs[a.index(1)] == self.sys[i][0]
                    rows.append(np.full(B, 1.0 if one else 0.0))
        return np.stack(rows) if rows else np.zeros((0, B))

    @property
    def has_time(self):
        """Whether the initial time is among the arguments (the initial values
        of the derivatives then depend on the state, the parameters and t0)."""
        return any(a.kind == _e.TIME for a in self.vargs)

    def initial_variational_state_at(self, x0, t0, pars=None):
        """The initial values of the derivatives for initial conditions x0
        (n_orig_sv, B) at times t0 (B,) with parameters pars (n_pars, B):
        the identity for state arguments at order 1, the Lie-derivative sums
        of the module docstring for derivatives that involve t0, zero
        otherwise.  Shape (n_derivatives, B)."""
        import numpy as np

        x0 = np.asarray(x0, dtype=np.float64)
        B = x0.shape[1]
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (B,))
        pars = None if pars is None else np.asarray(pars, dtype=np.float64)
        env = {x.value: x0[i] for i, (x, _) in enumerate(self._orig)}
        base = self.initial_variational_state(B)
        ti = [j for j, a in enumerate(self.vargs) if a.kind == _e.TIME]
        if not ti:
            return base
        ti = ti[0]
        xs = [x for x, _ in self._orig]
        fs = [f for _, f in self._orig]
        lie = {}  # (i, j) -> L^j(x_i)

        def L(i, j):
            if (i, j) not in lie:
                if j == 1:
                    lie[(i, j)] = fs[i]
                else:
                    g = L(i, j - 1)
                    terms = [_e.diff(g, x) * f for x, f in zip(xs, fs)]
                    terms.append(_e.diff_time(g))
                    lie[(i, j)] = _e.sum(terms)
            return lie[(i, j)]

        row = 0
        out = base.copy()
        for r in range(1, self.order + 1):
            for i in range(self.n_orig_sv):
                for a in self._mi[r]:
                    k = a[ti]
                    if k:
                        tot = np.zeros(B)
                        for j in range(1, k + 1):
                            g = L(i, j)
                            for _ in range(k - j):
                                g = _e.diff_time(g)
                            for q, c in enumerate(a):
                                if q != ti:
                                    for _ in range(c):
                                        g = _e.diff(g, self.vargs[q])
                            val = _e.evaluate(g, env, pars, t0)
                            tot = tot + math.comb(k, j) * (-1.0) ** j * np.broadcast_to(val, (B,))
                        out[row] = tot
                    row += 1
        return out

    def _count(self, r):
        return len(self._mi[r]) if r >= 1 else 1

    def vslice(self, order, component=None):
        n = self.n_orig_sv
        if order < 0 or order > self.order:
            raise ValueError("invalid variational order")
        if order == 0:
            return slice(0, n) if component is None else slice(component, component + 1)
        start = n + sum(n * self._count(r) for r in range(1, order))
        c = self._count(order)
        if component is None:
            return slice(start, start + n * c)
        if not 0 <= component < n:
            raise ValueError("invalid component")
        return slice(start + component * c, start + (component + 1) * c)

    def mindex(self, i):
        n, m = self.n_orig_sv, len(self.vargs)
        if i < n:
            return [i] + [0] * m
        k = i - n
        for r in range(1, self.order + 1):
            c = self._count(r)
            if k < n * c:
                comp, j = divmod(k, c)
                return [comp] + list(self._mi[r][j])
            k -= n * c
        raise ValueError("index out of range")

    def taylor_map_terms(self):
        """(state row, component, multi-index, 1/alpha!) for every term of the Taylor map."""
        out = []
        total = self.n_orig_sv + sum(self.n_orig_sv * self._count(r) for r in range(1, self.order + 1))
        for row in range(total):
            mi = self.mindex(row)
            a = mi[1:]
            fact = 1.0
            for x in a:
                fact *= math.factorial(x)
            out.append((row, mi[0], a, 1.0 / fact))
        return out
