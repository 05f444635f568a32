"""First-order variational equations: ``var_ode_sys(sys, args, order=1)``.

Restates the reference's variational ODE construction
(heyoka/expose_var_ode_sys.cpp:29-59, batch variational API
heyoka/expose_batch_integrators.cpp:549-649) at order 1: the system is
augmented with the sensitivities dx_i/d(arg_j) of every state variable with
respect to the chosen arguments (initial values of state variables and/or
runtime parameters),

    d/dt (dx_i/da_j) = sum_k (df_i/dx_k) (dx_k/da_j) + df_i/da_j,

with the layout the reference's tests pin (heyoka/_test_var_integrator.py:
190-201): the original state first, then for each component i and each
argument j in order, dx_i/da_j.  Initial values: the identity for state
arguments, zero for parameters.
"""

from __future__ import annotations

import enum

from . import expr as _e


class var_args(enum.IntFlag):
    vars = 1
    params = 2
    time = 4
    all = 7


class var_ode_sys:
    def __init__(self, sys, args=var_args.vars, order=1):
        if order != 1:
            raise NotImplementedError("only first-order variational equations are supported")
        pairs = [(_e._ex(l), _e._ex(r)) for l, r in sys]
        xs = [l for l, _ in pairs]
        if isinstance(args, var_args):
            if args & var_args.time:
                raise NotImplementedError("sensitivities with respect to the initial time are not supported")
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
        else:
            vargs = [_e._ex(a) for a in args]
            for a in vargs:
                if not (a.kind == _e.PAR or (a.kind == _e.VAR and a in xs)):
                    raise ValueError("variational arguments must be state variables or parameters")
        n, m = len(pairs), len(vargs)
        dvars = [[_e.make_vars("d_{}_{}".format(i, j)) for j in range(m)] for i in range(n)]
        jac = [[_e.diff(f, x) for x in xs] for _, f in pairs]
        out = list(pairs)
        for i, (_, f) in enumerate(pairs):
            for j, a in enumerate(vargs):
                terms = [jac[i][k] * dvars[k][j] for k in range(n)]
                if a.kind == _e.PAR:
                    terms.append(_e.diff(f, a))
                out.append((dvars[i][j], _e.sum(terms)))
        self.sys = out
        self.vargs = vargs
        self.n_orig_sv = n
        self.order = 1

    def initial_variational_state(self, B):
        """The (n * m, B) initial values of the sensitivities."""
        import numpy as np

        n, m = self.n_orig_sv, len(self.vargs)
        out = np.zeros((n * m, B))
        for i in range(n):
            for j, a in enumerate(self.vargs):
                if a.kind == _e.VAR and a == self.sys[i][0]:
                    out[i * m + j] = 1.0
        return out

    def vslice(self, order, component=None):
        n, m = self.n_orig_sv, len(self.vargs)
        if order == 0:
            return slice(0, n) if component is None else slice(component, component + 1)
        if order == 1:
            if component is None:
                return slice(n, n + n * m)
            return slice(n + component * m, n + (component + 1) * m)
        raise ValueError("invalid variational order")

    def mindex(self, i):
        n, m = self.n_orig_sv, len(self.vargs)
        if i < n:
            return [i] + [0] * m
        k = i - n
        comp, arg = divmod(k, m)
        out = [comp] + [0] * m
        out[1 + arg] = 1
        return out
