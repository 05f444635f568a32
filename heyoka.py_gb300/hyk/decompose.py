"""Taylor decomposition of an ODE system into elementary u-variables.

The reference exposes the decomposition of a batch integrator as a list of
``(expression, dependencies)`` entries: first the n state variables, then the
elementary operations in topological order, then the n right-hand sides
(heyoka/expose_batch_integrators.cpp:231, described in
doc/notebooks/sympy_interop.ipynb).  The decomposition itself happens inside
the heyoka C++ library; this module is an independent restatement with the
same layout and the same elementary-operation vocabulary:

* ``add sub mul div neg`` (binary / unary arithmetic),
* ``square`` (for ``x**2``), ``sqrt`` (for ``x**0.5`` and ``sqrt``),
  ``pow`` (numeric exponent),
* ``exp log``,
* ``sin``/``cos`` as a coupled pair: asking for either one adds both, sine
  first, each recording its partner (the reference couples them the same way,
  since each one's recurrence needs the other).

Common subexpressions are merged by structural hashing.  Numbers, runtime
parameters and the time variable are not u-variables; they appear as
operation arguments whose Taylor coefficients are known in closed form.

The result is flattened into the plain arrays of the C ABI declared in
``include/hyk.h`` (``hyk_arg_t`` / ``hyk_uop_t``), which the CUDA code
generator and the CPU oracle both consume.
"""

from __future__ import annotations

import ctypes
import hashlib
import struct
from dataclasses import dataclass, field

from . import expr as _e

# Keep in sync with include/hyk.h.
OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG = 0, 1, 2, 3, 4
OP_SQUARE, OP_SQRT, OP_POW, OP_EXP, OP_LOG = 5, 6, 7, 8, 9
OP_SIN, OP_COS = 10, 11

ARG_NONE, ARG_U, ARG_NUM, ARG_PAR, ARG_TIME = 0, 1, 2, 3, 4

OP_NAMES = {
    OP_ADD: "add",
    OP_SUB: "sub",
    OP_MUL: "mul",
    OP_DIV: "div",
    OP_NEG: "neg",
    OP_SQUARE: "square",
    OP_SQRT: "sqrt",
    OP_POW: "pow",
    OP_EXP: "exp",
    OP_LOG: "log",
    OP_SIN: "sin",
    OP_COS: "cos",
}
_NAME_TO_OP = {v: k for k, v in OP_NAMES.items()}


class hyk_arg_t(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("idx", ctypes.c_int32), ("num", ctypes.c_double)]


class hyk_uop_t(ctypes.Structure):
    _fields_ = [
        ("op", ctypes.c_int32),
        ("aux", ctypes.c_int32),
        ("a", hyk_arg_t),
        ("b", hyk_arg_t),
    ]


class hyk_event_t(ctypes.Structure):
    _fields_ = [
        ("g", hyk_arg_t),
        ("terminal", ctypes.c_int32),
        ("direction", ctypes.c_int32),
        ("cooldown", ctypes.c_double),
    ]


class hyk_decomp_t(ctypes.Structure):
    _fields_ = [
        ("n_eq", ctypes.c_uint32),
        ("n_ops", ctypes.c_uint32),
        ("n_pars", ctypes.c_uint32),
        ("n_ev", ctypes.c_uint32),
        ("ops", ctypes.POINTER(hyk_uop_t)),
        ("rhs", ctypes.POINTER(hyk_arg_t)),
        ("ev", ctypes.POINTER(hyk_event_t)),
    ]


Arg = tuple  # (kind, idx, num)


@dataclass
class Decomposition:
    """A flattened Taylor decomposition.

    ``ops[k]`` defines u-variable ``n_eq + k``; ``rhs[i]`` is the right-hand
    side of state variable ``i``.  Each op is ``(opcode, aux, a, b)`` with
    ``a``/``b`` arguments ``(kind, idx, num)``.
    """

    n_eq: int
    n_pars: int
    state_names: list
    ops: list = field(default_factory=list)
    rhs: list = field(default_factory=list)
    sys: list = field(default_factory=list)
    # events: (arg, terminal, direction, cooldown), non-terminal and terminal in one list
    ev: list = field(default_factory=list)

    @property
    def n_ops(self):
        return len(self.ops)

    @property
    def n_u(self):
        return self.n_eq + len(self.ops)

    def digest(self) -> str:
        """Stable hash of the decomposition (used as a compiled-module cache key)."""
        h = hashlib.sha256()
        h.update(struct.pack("<II", self.n_eq, self.n_pars))
        for op, aux, a, b in self.ops:
            h.update(struct.pack("<ii", op, aux))
            for k, i, v in (a, b):
                h.update(struct.pack("<iid", k, i, v))
        for k, i, v in self.rhs:
            h.update(struct.pack("<iid", k, i, v))
        for (k, i, v), term, dirn, cool in self.ev:
            h.update(struct.pack("<iidiid", k, i, v, int(term), int(dirn), float(cool)))
        return h.hexdigest()

    def as_c(self):
        """Return ``(hyk_decomp_t, keepalive)`` for passing through the C ABI."""
        n = len(self.ops)
        ops = (hyk_uop_t * max(n, 1))()
        for k, (op, aux, a, b) in enumerate(self.ops):
            ops[k].op, ops[k].aux = op, aux
            ops[k].a.kind, ops[k].a.idx, ops[k].a.num = a
            ops[k].b.kind, ops[k].b.idx, ops[k].b.num = b
        rhs = (hyk_arg_t * max(self.n_eq, 1))()
        for i, (k, j, v) in enumerate(self.rhs):
            rhs[i].kind, rhs[i].idx, rhs[i].num = k, j, v
        ev = (hyk_event_t * max(len(self.ev), 1))()
        for j, ((k, i, v), term, dirn, cool) in enumerate(self.ev):
            ev[j].g.kind, ev[j].g.idx, ev[j].g.num = k, i, v
            ev[j].terminal, ev[j].direction, ev[j].cooldown = int(term), int(dirn), float(cool)
        d = hyk_decomp_t()
        d.n_eq, d.n_ops, d.n_pars, d.n_ev = self.n_eq, n, self.n_pars, len(self.ev)
        d.ops = ctypes.cast(ops, ctypes.POINTER(hyk_uop_t))
        d.rhs = ctypes.cast(rhs, ctypes.POINTER(hyk_arg_t))
        d.ev = ctypes.cast(ev, ctypes.POINTER(hyk_event_t)) if self.ev else None
        return d, (ops, rhs, ev)

    # Pretty form mirroring the reference's ``decomposition`` property.
    def as_list(self):
        out = []
        for i, name in enumerate(self.state_names):
            out.append((_e.expression(name), []))
        for op, aux, a, b in self.ops:
            args = [a] if b[0] == ARG_NONE else [a, b]
            deps = sorted(x[1] for x in args if x[0] == ARG_U)
            out.append((_op_str(op, a, b, self), deps))
        for r in self.rhs:
            out.append((_arg_str(r, self), [r[1]] if r[0] == ARG_U else []))
        return out


def _arg_str(a, d):
    k, i, v = a
    if k == ARG_U:
        return "u_{}".format(i)
    if k == ARG_NUM:
        return repr(v)
    if k == ARG_PAR:
        return "p{}".format(i)
    if k == ARG_TIME:
        return "t"
    return ""


def _op_str(op, a, b, d):
    name = OP_NAMES[op]
    if b[0] == ARG_NONE:
        return "{}({})".format(name, _arg_str(a, d))
    return "{}({}, {})".format(name, _arg_str(a, d), _arg_str(b, d))


_NONE: Arg = (ARG_NONE, 0, 0.0)


def taylor_decompose(sys, events=()) -> Decomposition:
    """Decompose ``sys = [(x0, rhs0), (x1, rhs1), ...]`` into u-variables.

    ``events``: ``(expression, terminal, direction, cooldown)`` tuples; the
    event functions are decomposed together with the system (shared
    subexpressions are computed once), like the reference's event equations."""
    try:
        pairs = [(_e._ex(l), _e._ex(r)) for l, r in sys]
    except (TypeError, ValueError) as exc:
        raise TypeError(
            "The system of ODEs must be a list of (variable, expression) pairs"
        ) from exc
    if len(pairs) == 0:
        raise ValueError("Cannot integrate a system of ODEs with zero equations")

    names = []
    for l, _ in pairs:
        if l.kind != _e.VAR:
            raise ValueError(
                "Invalid system of differential equations detected: the "
                "left-hand side contains the expression '{}', which is not a variable".format(l)
            )
        if l.value in names:
            raise ValueError(
                "Invalid system of differential equations detected: the variable '{}' "
                "appears in the left-hand side twice".format(l.value)
            )
        names.append(l.value)
    index = {n: i for i, n in enumerate(names)}
    n_eq = len(names)

    ops: list = []
    memo: dict = {}
    sincos: dict = {}
    n_pars = 0

    def add_op(op, a, b=_NONE, aux=-1):
        ops.append((op, aux, a, b))
        return n_eq + len(ops) - 1

    def visit(node) -> Arg:
        nonlocal n_pars
        if node.kind == _e.VAR:
            if node.value not in index:
                raise ValueError(
                    "Invalid system of differential equations detected: the variable '{}' "
                    "appears in the right-hand side but it is not a state variable".format(node.value)
                )
            return (ARG_U, index[node.value], 0.0)
        if node.kind == _e.NUM:
            return (ARG_NUM, 0, node.value)
        if node.kind == _e.PAR:
            n_pars = max(n_pars, node.value + 1)
            return (ARG_PAR, node.value, 0.0)
        if node.kind == _e.TIME:
            return (ARG_TIME, 0, 0.0)
        if node in memo:
            return memo[node]
        name = node.value
        args = [visit(a) for a in node.args]
        if name in ("sin", "cos"):
            key = args[0]
            if key not in sincos:
                s = add_op(OP_SIN, key)
                c = add_op(OP_COS, key)
                ops[s - n_eq] = (OP_SIN, c, key, _NONE)
                ops[c - n_eq] = (OP_COS, s, key, _NONE)
                sincos[key] = (s, c)
            u = sincos[key][0 if name == "sin" else 1]
        elif name == "pow":
            alpha = args[1][2]
            if alpha == 2.0:
                u = add_op(OP_SQUARE, args[0])
            elif alpha == 0.5:
                u = add_op(OP_SQRT, args[0])
            else:
                u = add_op(OP_POW, args[0], (ARG_NUM, 0, alpha))
        elif name in ("neg", "square", "sqrt", "exp", "log"):
            u = add_op(_NAME_TO_OP[name], args[0])
        else:
            u = add_op(_NAME_TO_OP[name], args[0], args[1])
        ret = (ARG_U, u, 0.0)
        memo[node] = ret
        return ret

    rhs = [visit(r) for _, r in pairs]
    ev = []
    for ex, term, dirn, cool in events:
        ex = _e._ex(ex)
        for name in _e.get_variables(ex):
            if name not in index:
                raise ValueError(
                    "The event expression '{}' contains the variable '{}', which is not a state variable".format(ex, name)
                )
        ev.append((visit(ex), bool(term), int(dirn), float(cool)))
    return Decomposition(n_eq=n_eq, n_pars=n_pars, state_names=names, ops=ops, rhs=rhs, sys=pairs, ev=ev)


def order_from_tol(tol: float) -> int:
    """Taylor order for a tolerance: ceil(-ln(tol)/2 + 1).

    This is the Jorba-Zou order rule used by the reference (heyoka MNRAS 2021
    paper cited in README.md:61-63); it reproduces the reference's order 20 at
    tol = 2.22e-16 (doc/notebooks/The adaptive integrator.ipynb, cell 1) and
    12 at tol = 1e-9 (doc/notebooks/Customising the adaptive integrator.ipynb).
    """
    import math

    if not (tol > 0.0) or not math.isfinite(tol):
        raise ValueError(
            "The tolerance in an adaptive Taylor integrator must be finite and positive, "
            "but it is {} instead".format(tol)
        )
    order = math.ceil(-math.log(tol) / 2.0 + 1.0)
    if order < 2:
        raise ValueError(
            "The Taylor order deduced from the tolerance ({}) is less than 2".format(order)
        )
    return int(order)
