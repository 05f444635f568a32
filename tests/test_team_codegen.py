"""The team form's recurrences on the CPU.

The code generator's team form (several threads per trajectory, the
u-operations of a dependency level spread over the team, orders as a runtime
loop over per-operation descriptors) is built for the host as a team of one
thread and stepped once; the result must equal the oracle's gpu-arithmetic
step bit for bit, for systems that cover every operation and operand kind the
team form accepts (variables, numbers, parameters, the time)."""

import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

import hyk
from hyk import _lib, workloads as W
from hyk.decompose import taylor_decompose

pd = ctypes.POINTER(ctypes.c_double)


def _team_host(libhyk, sys_, order, team=2):
    d, keep = taylor_decompose(sys_).as_c()
    cfg = _lib.hyk_config_t(0, 0, 0, team)
    buf = ctypes.create_string_buffer(1 << 24)
    rc = libhyk.hyk_codegen_check(ctypes.byref(d), order, ctypes.byref(cfg), 3, buf, len(buf), None, None)
    assert rc == 0, libhyk.hyk_last_error()
    tmp = tempfile.mkdtemp()
    src, so = os.path.join(tmp, "t.cpp"), os.path.join(tmp, "t.so")
    with open(src, "w") as f:
        f.write(buf.value.decode())
    subprocess.run(["g++", "-O1", "-ffp-contract=off", "-shared", "-fPIC", src, "-o", so], check=True)
    return ctypes.CDLL(so)


def _mixed():
    x, y = hyk.make_vars("x", "y")
    t, p = hyk.time, hyk.par
    return [
        (x, hyk.exp(-y) * hyk.log(x) + hyk.sqrt(y) / x + hyk.cos(t) * p[1] + p[0] / y + x * t + 0.5 * t),
        (y, p[0] / (x + 2.0) - x**-1.5 * p[1] + hyk.sin(x) * y + hyk.square(x - y) + t * y - (3.0 - x)
         + hyk.exp(t) * 1e-3 + y**2.5 + (x - t) / 7.0 + 2.0 - t),
    ]


def _consts():
    # time-constant operations (only an order-0 value) feeding every kind of operation
    x, y = hyk.make_vars("x", "y")
    p = hyk.par
    c1, c2 = 1.0 - p[0], hyk.exp(p[1])
    return [
        (x, c1 * y + c2 * hyk.sin(x) + hyk.sqrt(p[0] + 2.0) - (p[0] * 3.0) / (x + 4.0) + y / (p[1] + 1.0)),
        (y, -x * hyk.sin(p[1]) + hyk.cos(p[0] * x) + (c1 - y) ** 2.0 + hyk.log(c2 + x * x) - c1),
    ]


def _var2():
    from hyk import var

    x, v = hyk.make_vars("x", "v")
    orig = [(x, v), (v, hyk.cos(hyk.time) - hyk.par[0] * v - hyk.sin(x))]
    return var.var_ode_sys(orig, var.var_args.vars | var.var_args.params, order=2)


CASES = {
    "pendulum": lambda: (W.pendulum_sys(), W.pendulum_ics(3, seed=1), None, 20),
    "kepler": lambda: (W.kepler_sys(), W.kepler_ics(3, seed=2), None, 19),
    "cr3bp": lambda: (W.cr3bp_sys(),) + W.cr3bp_ics(3, seed=3) + (19,),
    "oss": lambda: (W.oss_sys(), W.oss_ics(3, seed=4)[0], None, 19),
    "mixed": lambda: (_mixed(), np.array([[1.1, 0.9, 1.3], [0.8, 0.7, 1.2]]), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6]]), 12),
    "var2": lambda: (_var2().sys, np.concatenate([np.array([[0.2, 0.21], [0.3, 0.31]]), _var2().initial_variational_state(2)]),
                     np.array([[0.4, 0.41]]), 20),
    "consts": lambda: (_consts(), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6]]), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6]]), 15),
}


@pytest.mark.parametrize("form", ["team", "lane"])
@pytest.mark.parametrize("name", list(CASES))
def test_team_recurrences_bitwise_vs_oracle(libhyk, oracle, name, form):
    """Both forms' generated recurrences (lane form: the host build of the
    per-lane code; team form: a team of one) against the oracle."""
    sys_, st, pars, order = CASES[name]()
    H = _team_host(libhyk, sys_, order, team=2 if form == "team" else 1)
    o = oracle.Oracle(sys_, st, pars=pars, order=order, mode=1, time=np.full(st.shape[1], 0.25))
    _, h = o.step()
    S = np.zeros(H.hyk_host_nslot())
    n_eq = st.shape[0]
    for lane in range(st.shape[1]):
        x0 = np.ascontiguousarray(st[:, lane], dtype=np.float64)
        p = np.ascontiguousarray(pars[:, lane] if pars is not None else np.zeros(1), dtype=np.float64)
        x1 = np.zeros(len(x0))
        H.hyk_host_step(S.ctypes.data_as(pd), x0.ctypes.data_as(pd), p.ctypes.data_as(pd), ctypes.c_double(0.25),
                        ctypes.c_double(h[lane]), x1.ctypes.data_as(pd))
        assert np.array_equal(x1, o.state[:, lane]), (name, lane)
        # Every Taylor coefficient, not only the stepped state (whose Horner
        # sum can hide last-bit differences of the high orders).
        tc = np.zeros(n_eq * (order + 1))
        H.hyk_host_tc(S.ctypes.data_as(pd), x0.ctypes.data_as(pd), p.ctypes.data_as(pd), ctypes.c_double(0.25),
                      tc.ctypes.data_as(pd))
        assert np.array_equal(tc.reshape(n_eq, order + 1), o.tc[:, :, lane]), (name, lane)


def test_team_form_rejects_unsupported_operand(libhyk):
    # pow of the time itself has no team-form code (the lane form handles it)
    x, v = hyk.make_vars("x", "v")
    d, keep = taylor_decompose([(x, v), (v, hyk.time**2.0 * x)]).as_c()
    cfg = _lib.hyk_config_t(0, 0, 0, 4)
    rc = libhyk.hyk_codegen_check(ctypes.byref(d), 10, ctypes.byref(cfg), 2, None, 0, None, None)
    assert rc != 0 and b"non-variable argument" in libhyk.hyk_last_error()
    cfg = _lib.hyk_config_t(0, 0, 0, 1)
    assert libhyk.hyk_codegen_check(ctypes.byref(d), 10, ctypes.byref(cfg), 2, None, 0, None, None) == 0
