"""Symbolic expressions for ODE right-hand sides.

This is the input surface of the batch integrator: a small, immutable,
hash-consed expression graph with the constructors heyoka.py exposes
(``make_vars``, ``par``, ``time``, arithmetic operators, ``sin``, ``cos``,
``exp``, ``log``, ``sqrt``, ``square``, ``sum``).  It mirrors the behaviour of
the reference's expression class (heyoka/expose_expression.cpp:89-228 for the
operators, :260-277 for make_vars, :282-306 for the elementary functions,
heyoka/__init__.py:346-374 for ``par`` and ``time``) but is an independent
Python implementation: the reference's own expression system lives in the
heyoka C++ library, which is not part of this package.

Constant folding follows the conventions visible in the reference's tests
(heyoka/_test_model.py:153-166): operations between numbers fold into a
number, ``x * 0`` folds to ``0``, ``x * 1`` to ``x`` and ``x + 0`` to ``x``.
"""

from __future__ import annotations

import math
import numbers

__all__ = [
    "expression",
    "make_vars",
    "par",
    "time",
    "sin",
    "cos",
    "exp",
    "log",
    "sqrt",
    "square",
    "sum",
    "prod",
]

# Node kinds.
VAR, NUM, PAR, TIME, FUNC = "var", "num", "par", "time", "func"

# Elementary functions understood by the decomposer.
FUNCS = (
    "add",
    "sub",
    "mul",
    "div",
    "neg",
    "square",
    "sqrt",
    "pow",
    "exp",
    "log",
    "sin",
    "cos",
)


def _num_key(v: float):
    # Distinguish 0.0 from -0.0 and keep NaN hashable.
    return ("f", math.copysign(1.0, v), abs(v)) if v == v else ("nan",)


class expression:
    """An immutable symbolic expression node.

    ``expression(1.5)`` builds a number, ``expression("x")`` a variable,
    mirroring the reference's constructors (heyoka/expose_expression.cpp:89-120).
    """

    __slots__ = ("kind", "value", "args", "_hash")

    def __init__(self, value=0.0, *, _kind=None, _args=()):
        if _kind is None:
            if isinstance(value, expression):
                _kind, _args, value = value.kind, value.args, value.value
            elif isinstance(value, str):
                _kind = VAR
            elif isinstance(value, numbers.Real):
                _kind, value = NUM, float(value)
            else:
                raise TypeError(
                    "Cannot construct an expression from an object of type {}".format(type(value))
                )
        object.__setattr__(self, "kind", _kind)
        object.__setattr__(self, "value", value)
        object.__setattr__(self, "args", tuple(_args))
        key = (_kind, _num_key(value) if _kind == NUM else value, self.args)
        object.__setattr__(self, "_hash", hash(key))

    def __setattr__(self, *a):
        raise AttributeError("expressions are immutable")

    # Structural identity.
    def _key(self):
        return (
            self.kind,
            _num_key(self.value) if self.kind == NUM else self.value,
            tuple(a._key() for a in self.args),
        )

    def __hash__(self):
        return self._hash

    def __eq__(self, other):
        if not isinstance(other, expression):
            try:
                other = _ex(other)
            except TypeError:
                return NotImplemented
        if self is other:
            return True
        if self._hash != other._hash or self.kind != other.kind:
            return False
        if self.kind == NUM:
            return _num_key(self.value) == _num_key(other.value)
        return self.value == other.value and self.args == other.args

    def __ne__(self, other):
        r = self.__eq__(other)
        return r if r is NotImplemented else not r

    # Arithmetic.
    def __add__(self, o):
        return _add(self, _ex(o))

    def __radd__(self, o):
        return _add(_ex(o), self)

    def __sub__(self, o):
        return _sub(self, _ex(o))

    def __rsub__(self, o):
        return _sub(_ex(o), self)

    def __mul__(self, o):
        return _mul(self, _ex(o))

    def __rmul__(self, o):
        return _mul(_ex(o), self)

    def __truediv__(self, o):
        return _div(self, _ex(o))

    def __rtruediv__(self, o):
        return _div(_ex(o), self)

    def __neg__(self):
        return _neg(self)

    def __pos__(self):
        return self

    def __pow__(self, o):
        return _pow(self, _ex(o))

    def __rpow__(self, o):
        return _pow(_ex(o), self)

    # Introspection helpers.
    @property
    def is_number(self):
        return self.kind == NUM

    def __float__(self):
        if self.kind != NUM:
            raise TypeError("Only numerical expressions can be converted to float")
        return self.value

    def __repr__(self):
        return _str(self)

    __str__ = __repr__

    def __copy__(self):
        return self

    def __deepcopy__(self, memo):
        return self

    def __reduce__(self):
        return (_rebuild, (self.kind, self.value, self.args))


def _rebuild(kind, value, args):
    return expression(value, _kind=kind, _args=args)


def _ex(x) -> expression:
    if isinstance(x, expression):
        return x
    if isinstance(x, numbers.Real) and not isinstance(x, bool):
        return expression(float(x))
    if isinstance(x, bool):
        return expression(float(x))
    # numpy scalars
    try:
        import numpy as _np

        if isinstance(x, _np.generic) and _np.issubdtype(type(x), _np.floating):
            return expression(float(x))
    except ImportError:  # pragma: no cover
        pass
    raise TypeError("Cannot convert an object of type {} to an expression".format(type(x)))


def _func(name, *args):
    return expression(name, _kind=FUNC, _args=args)


def _isnum(e, v=None):
    return e.kind == NUM and (v is None or e.value == v)


def _add(a, b):
    if _isnum(a) and _isnum(b):
        return expression(a.value + b.value)
    if _isnum(a, 0.0):
        return b
    if _isnum(b, 0.0):
        return a
    return _func("add", a, b)


def _sub(a, b):
    if _isnum(a) and _isnum(b):
        return expression(a.value - b.value)
    if _isnum(b, 0.0):
        return a
    if _isnum(a, 0.0):
        return _neg(b)
    return _func("sub", a, b)


def _mul(a, b):
    if _isnum(a) and _isnum(b):
        return expression(a.value * b.value)
    if _isnum(a, 0.0) or _isnum(b, 0.0):
        return expression(0.0)
    if _isnum(a, 1.0):
        return b
    if _isnum(b, 1.0):
        return a
    return _func("mul", a, b)


def _div(a, b):
    if _isnum(a) and _isnum(b):
        return expression(a.value / b.value)
    if _isnum(b, 1.0):
        return a
    if _isnum(a, 0.0):
        return expression(0.0)
    return _func("div", a, b)


def _neg(a):
    if _isnum(a):
        return expression(-a.value)
    if a.kind == FUNC and a.value == "neg":
        return a.args[0]
    return _func("neg", a)


def _pow(a, b):
    if _isnum(a) and _isnum(b):
        return expression(math.pow(a.value, b.value))
    if not _isnum(b):
        raise NotImplementedError(
            "Only numerical exponents are supported by the GPU batch integrator"
        )
    e = b.value
    if e == 0.0:
        return expression(1.0)
    if e == 1.0:
        return a
    return _func("pow", a, b)


def make_vars(*names):
    """Create symbolic variables (reference: heyoka/expose_expression.cpp:260-277)."""
    if len(names) == 0:
        raise ValueError("At least one argument is required when invoking 'make_vars()'")
    ret = tuple(expression(str(n)) for n in names)
    return ret[0] if len(ret) == 1 else ret


class _par_generator:
    """``par[i]`` builds the runtime parameter at index i (heyoka/__init__.py:346-361)."""

    def __getitem__(self, idx):
        idx = int(idx)
        if idx < 0:
            raise ValueError("Parameter indices must be non-negative")
        return expression(idx, _kind=PAR)

    def __repr__(self):
        return "par"


par = _par_generator()
time = expression("t", _kind=TIME)


def sin(x):
    x = _ex(x)
    if _isnum(x):
        return expression(math.sin(x.value))
    return _func("sin", x)


def cos(x):
    x = _ex(x)
    if _isnum(x):
        return expression(math.cos(x.value))
    return _func("cos", x)


def exp(x):
    x = _ex(x)
    if _isnum(x):
        return expression(math.exp(x.value))
    return _func("exp", x)


def log(x):
    x = _ex(x)
    if _isnum(x):
        return expression(math.log(x.value))
    return _func("log", x)


def sqrt(x):
    x = _ex(x)
    if _isnum(x):
        return expression(math.sqrt(x.value))
    return _func("sqrt", x)


def square(x):
    x = _ex(x)
    if _isnum(x):
        return expression(x.value * x.value)
    return _func("square", x)


def sum(terms):  # noqa: A001 - mirrors the reference's name (expose_expression.cpp:282)
    """Left-to-right sum of a list of expressions."""
    terms = [_ex(t) for t in terms]
    if not terms:
        return expression(0.0)
    acc = terms[0]
    for t in terms[1:]:
        acc = acc + t
    return acc


def prod(terms):
    """Left-to-right product of a list of expressions."""
    terms = [_ex(t) for t in terms]
    if not terms:
        return expression(1.0)
    acc = terms[0]
    for t in terms[1:]:
        acc = acc * t
    return acc


_BIN = {"add": "+", "sub": "-", "mul": "*", "div": "/"}


def _str(e: expression) -> str:
    if e.kind == VAR:
        return e.value
    if e.kind == NUM:
        return "{:.16f}".format(e.value) if math.isfinite(e.value) else repr(e.value)
    if e.kind == PAR:
        return "p{}".format(e.value)
    if e.kind == TIME:
        return "t"
    name, args = e.value, e.args
    if name in _BIN:
        return "({} {} {})".format(_str(args[0]), _BIN[name], _str(args[1]))
    if name == "neg":
        return "-{}".format(_str(args[0]))
    if name == "pow":
        return "{}**{}".format(_str(args[0]), _str(args[1]))
    return "{}({})".format(name, ", ".join(_str(a) for a in args))


def get_variables(e) -> list:
    """Sorted list of the variable names appearing in an expression or list of them."""
    out = set()
    stack = list(e) if isinstance(e, (list, tuple)) else [e]
    while stack:
        n = stack.pop()
        if n.kind == VAR:
            out.add(n.value)
        stack.extend(n.args)
    return sorted(out)


def diff(e, v):
    """Symbolic derivative of ``e`` with respect to a variable or parameter
    (reference: heyoka/expose_expression.cpp:531)."""
    e, v = _ex(e), _ex(v)
    if v.kind not in (VAR, PAR):
        raise ValueError("Derivatives can be taken only with respect to variables or parameters")
    return _deriv(e, v)


def diff_time(e):
    """Partial derivative of ``e`` with respect to the explicit time."""
    return _deriv(_ex(e), time)


def _deriv(e, v):
    memo = {}

    def d(n):
        if n in memo:
            return memo[n]
        if n.kind in (VAR, PAR, TIME):
            r = expression(1.0) if n == v else expression(0.0)
        elif n.kind == NUM:
            r = expression(0.0)
        else:
            f, a = n.value, n.args
            if f == "add":
                r = d(a[0]) + d(a[1])
            elif f == "sub":
                r = d(a[0]) - d(a[1])
            elif f == "neg":
                r = -d(a[0])
            elif f == "mul":
                r = d(a[0]) * a[1] + a[0] * d(a[1])
            elif f == "div":
                r = d(a[0]) / a[1] - a[0] * d(a[1]) / square(a[1])
            elif f == "square":
                r = 2.0 * a[0] * d(a[0])
            elif f == "sqrt":
                r = d(a[0]) / (2.0 * n)
            elif f == "pow":
                alpha = a[1].value
                r = alpha * a[0] ** (alpha - 1.0) * d(a[0])
            elif f == "exp":
                r = n * d(a[0])
            elif f == "log":
                r = d(a[0]) / a[0]
            elif f == "sin":
                r = cos(a[0]) * d(a[0])
            elif f == "cos":
                r = -(sin(a[0]) * d(a[0]))
            else:  # pragma: no cover
                raise NotImplementedError(f)
        memo[n] = r
        return r

    return d(e)


def evaluate(e, variables, pars=None, t=None):
    """Numerical value of ``e`` (NumPy, elementwise over lanes): ``variables``
    maps variable names to values, ``pars`` is indexable by parameter index,
    ``t`` is the time."""
    import numpy as np

    memo = {}
    stack = [(_ex(e), False)]
    while stack:
        n, ready = stack.pop()
        if n in memo:
            continue
        if n.kind == NUM:
            memo[n] = np.float64(n.value)
        elif n.kind == VAR:
            memo[n] = np.asarray(variables[n.value], dtype=np.float64)
        elif n.kind == PAR:
            memo[n] = np.asarray(pars[n.value], dtype=np.float64)
        elif n.kind == TIME:
            memo[n] = np.asarray(t, dtype=np.float64)
        elif not ready:
            stack.append((n, True))
            stack.extend((a, False) for a in n.args if a not in memo)
        else:
            a = [memo[x] for x in n.args]
            f = n.value
            if f == "add":
                r = a[0] + a[1]
            elif f == "sub":
                r = a[0] - a[1]
            elif f == "mul":
                r = a[0] * a[1]
            elif f == "div":
                r = a[0] / a[1]
            elif f == "neg":
                r = -a[0]
            elif f == "square":
                r = a[0] * a[0]
            elif f == "sqrt":
                r = np.sqrt(a[0])
            elif f == "pow":
                r = np.power(a[0], a[1])
            elif f == "exp":
                r = np.exp(a[0])
            elif f == "log":
                r = np.log(a[0])
            elif f == "sin":
                r = np.sin(a[0])
            elif f == "cos":
                r = np.cos(a[0])
            else:  # pragma: no cover
                raise NotImplementedError(f)
            memo[n] = r
    return memo[_ex(e)]
