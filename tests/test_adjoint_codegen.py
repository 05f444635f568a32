"""The generated reverse sweep on the CPU: the code generator's host build of
one Taylor step and of its adjoint, checked against central finite
differences of the step map (state and parameters).  This checks the adjoint
recurrences of every elementary operation without a GPU."""

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


def _host(libhyk, sys_, order):
    d, keep = taylor_decompose(sys_).as_c()
    cfg = _lib.hyk_config_t(0, 0, _lib.HYK_CFG_ADJOINT, 0)
    buf = ctypes.create_string_buffer(1 << 24)
    rc = libhyk.hyk_codegen_check(ctypes.byref(d), order, ctypes.byref(cfg), 3, buf, len(buf), None, None)
    assert rc == 0, libhyk.hyk_last_error()
    tmp = tempfile.mkdtemp()
    src, so = os.path.join(tmp, "h.cpp"), os.path.join(tmp, "h.so")
    with open(src, "w") as f:
        f.write(buf.value.decode())
    subprocess.run(["g++", "-O1", "-ffp-contract=off", "-shared", "-fPIC", src, "-o", so], check=True)
    return ctypes.CDLL(so)


def _arr(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(pd)


def _check(H, x0, pars, t0, h):
    S = np.zeros(H.hyk_host_nslot())
    n, P = len(x0), len(pars)
    pars = np.asarray(pars, dtype=np.float64)

    def step(x, p):
        x1 = np.zeros(n)
        H.hyk_host_step(_arr(S), _arr(x), _arr(p), ctypes.c_double(t0), ctypes.c_double(h), x1.ctypes.data_as(pd))
        return x1

    lam0 = np.random.default_rng(0).normal(size=n)
    lam, pb = lam0.copy(), np.zeros(max(P, 1))
    H.hyk_host_adjoint(_arr(S), _arr(x0), _arr(pars), ctypes.c_double(t0), ctypes.c_double(h),
                       lam.ctypes.data_as(pd), pb.ctypes.data_as(pd))
    fd = np.zeros(n)
    for i in range(n):
        e = 1e-6 * max(1.0, abs(x0[i]))
        a, b = np.array(x0, float), np.array(x0, float)
        a[i] += e
        b[i] -= e
        fd[i] = lam0 @ (step(a, pars) - step(b, pars)) / (2 * e)
    assert np.max(np.abs(lam - fd)) / np.max(np.abs(fd)) < 1e-8
    for k in range(P):
        e = 1e-6 * max(1.0, abs(pars[k]))
        a, b = pars.copy(), pars.copy()
        a[k] += e
        b[k] -= e
        fdp = lam0 @ (step(x0, a) - step(x0, b)) / (2 * e)
        assert abs(pb[k] - fdp) / max(abs(fdp), 1e-12) < 1e-7


def test_adjoint_step_pendulum_kepler_cr3bp(libhyk):
    x, v = hyk.make_vars("x", "v")
    _check(_host(libhyk, [(x, v), (v, -9.8 * hyk.sin(x))], 20), [0.3, 0.2], [], 0.0, 0.2)
    _check(_host(libhyk, W.kepler_sys(), 19), W.kepler_ics(1, seed=3)[:, 0], [], 0.0, 0.1)
    st, mu = W.cr3bp_ics(1, seed=3)
    _check(_host(libhyk, W.cr3bp_sys(), 19), st[:, 0], mu[:, 0], 0.0, 0.5)


def test_adjoint_step_every_operation(libhyk):
    x, y = hyk.make_vars("x", "y")
    sys_ = [
        (x, hyk.exp(-y) * hyk.log(x) + hyk.sqrt(y) / x + hyk.cos(hyk.time) * hyk.par[1] + hyk.par[0] / y),
        (y, hyk.par[0] / (x + 2.0) - x**-1.5 * hyk.par[1] + hyk.sin(x) * y + hyk.square(x - y) + hyk.par[1] * x),
    ]
    _check(_host(libhyk, sys_, 12), [1.1, 0.8], [0.3, 0.5], 0.4, 0.05)


def test_adjoint_step_scaled_sums(libhyk):
    """Sums of scaled terms computed as one chain (a difference, a negation,
    four terms and a fifth added to them) and the 6-body problem whose
    accelerations they are."""
    x, y, z = hyk.make_vars("x", "y", "z")
    sys_ = [
        (x, 2.0 * y - 3.0 * z),
        (y, -(4.0 * x) + z * x),
        (z, 0.5 * (x * y) + 0.25 * (y * z) - 0.125 * (z * x) + 1.5 * hyk.square(y) + 0.75 * x),
    ]
    _check(_host(libhyk, sys_, 12), [0.3, -0.2, 0.5], [], 0.0, 0.1)
    st, _ = W.oss_ics(1, seed=4)
    _check(_host(libhyk, W.oss_sys(), 19), st[:, 0], [], 0.0, 50.0)


def test_per_order_functions_bitwise_vs_oracle(libhyk, oracle):
    """A system large enough for the one-function-per-order form (5-body
    problem, 160 u-operations at order 19): the host build of the generated
    step agrees bit for bit with the oracle's gpu-arithmetic step."""
    sys_ = hyk.model.nbody(5)
    d, keep = taylor_decompose(sys_).as_c()
    cfg = _lib.hyk_config_t(0, 0, 0, 0)
    buf = ctypes.create_string_buffer(1 << 24)
    assert libhyk.hyk_codegen_check(ctypes.byref(d), 19, ctypes.byref(cfg), 3, buf, len(buf), None, None) == 0
    src = buf.value.decode()
    assert "hyk_jets_o18" in src
    tmp = tempfile.mkdtemp()
    f, so = os.path.join(tmp, "h.cpp"), os.path.join(tmp, "h.so")
    with open(f, "w") as fh:
        fh.write(src)
    subprocess.run(["g++", "-O1", "-ffp-contract=off", "-shared", "-fPIC", f, "-o", so], check=True)
    H = ctypes.CDLL(so)
    st = np.random.default_rng(5).normal(size=(30, 3))
    o = oracle.Oracle(sys_, st, order=19, mode=1)
    _, h = o.step()
    S = np.zeros(H.hyk_host_nslot())
    for lane in range(3):
        x1 = np.zeros(30)
        H.hyk_host_step(_arr(S), _arr(st[:, lane]), _arr(np.zeros(1)), ctypes.c_double(0.0), ctypes.c_double(h[lane]),
                        x1.ctypes.data_as(pd))
        assert np.array_equal(x1, o.state[:, lane])
        tc = np.zeros(30 * 20)
        H.hyk_host_tc(_arr(S), _arr(st[:, lane]), _arr(np.zeros(1)), ctypes.c_double(0.0), tc.ctypes.data_as(pd))
        assert np.array_equal(tc.reshape(30, 20), o.tc[:, :, lane])
