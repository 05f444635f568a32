"""hyk - GB300-native batch Taylor integrator with heyoka.py's batch API."""
from .expr import expression, make_vars, par, time, sin, cos, exp, log, sqrt, square, sum, prod  # noqa: F401
from .decompose import taylor_decompose, order_from_tol  # noqa: F401
from . import model  # noqa: F401
