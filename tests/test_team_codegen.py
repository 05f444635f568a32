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
import systems
from hyk import _lib, workloads as W
from hyk.decompose import taylor_decompose

pd = ctypes.POINTER(ctypes.c_double)


def _team_host(libhyk, sys_, order, team=2, flags=0):
    d, keep = taylor_decompose(sys_).as_c()
    cfg = _lib.hyk_config_t(0, 0, flags, team)
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
    return systems.mixed()


def _consts():
    return systems.consts()


def _var2():
    return systems.var2()


CASES = {
    "pendulum": lambda: (W.pendulum_sys(), W.pendulum_ics(3, seed=1), None, 20),
    "kepler": lambda: (W.kepler_sys(), W.kepler_ics(3, seed=2), None, 19),
    "cr3bp": lambda: (W.cr3bp_sys(),) + W.cr3bp_ics(3, seed=3) + (19,),
    "oss": lambda: (W.oss_sys(), W.oss_ics(3, seed=4)[0], None, 19),
    "mixed": lambda: (_mixed(), np.array([[1.1, 0.9, 1.3], [0.8, 0.7, 1.2]]), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6]]), 12),
    "var2": lambda: (_var2().sys, np.concatenate([np.array([[0.2, 0.21], [0.3, 0.31]]), _var2().initial_variational_state(2)]),
                     np.array([[0.4, 0.41]]), 20),
    "consts": lambda: (_consts(), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6]]), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6]]), 15),
    # every state variable read at its current order only (cold state rows
    # in the team form), x' = v among the updates, j x_j of a cold variable
    "linear": lambda: (_linear(), np.array([[0.3, 0.2, 0.1], [0.5, 0.4, 0.6], [-0.2, 0.1, 0.3], [0.7, -0.5, 0.2]]), None, 14),
}


def _linear():
    x, v, y, w = hyk.make_vars("x", "v", "y", "w")
    # (sin(x) reads the j x_j of x, not its orders)
    return [(x, v), (v, -2.0 * x + 0.5 * y - 0.25 * v), (y, w), (w, -y + 0.3 * x + 1.5 * hyk.sin(x))]


@pytest.mark.parametrize("form", ["team", "team_hot", "lane"])
@pytest.mark.parametrize("name", list(CASES))
def test_team_recurrences_bitwise_vs_oracle(libhyk, oracle, name, form):
    """Both forms' generated recurrences (lane form: the host build of the
    per-lane code; team form: a team of one, with cold state rows where the
    system allows them, and without) against the oracle."""
    sys_, st, pars, order = CASES[name]()
    H = _team_host(libhyk, sys_, order, team=1 if form == "lane" else 2,
                   flags=_lib.HYK_CFG_NO_COLD_ROWS if form == "team_hot" else 0)
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


def test_cold_state_rows_layout(libhyk):
    """The team form keeps two shared-memory slots per state variable when
    every state variable is read at its current order only (6-body problem,
    the linear system), and p + 1 otherwise (Kepler's positions are squared)."""
    def slots(sys_, flags):
        d, keep = taylor_decompose(sys_).as_c()
        cfg = _lib.hyk_config_t(0, 0, flags, 16)
        n = ctypes.c_uint32()
        assert libhyk.hyk_codegen_check(ctypes.byref(d), 19, ctypes.byref(cfg), 2, None, 0, ctypes.byref(n), None) == 0
        return n.value

    for sys_, n_eq in ((W.oss_sys(), 36), (_linear(), 4)):
        hot, cold = slots(sys_, _lib.HYK_CFG_NO_COLD_ROWS), slots(sys_, 0)
        assert hot - cold == n_eq * (21 - 2), (hot, cold)
    k = W.kepler_sys()
    assert slots(k, 0) == slots(k, _lib.HYK_CFG_NO_COLD_ROWS)
