"""Single-precision recurrences on the CPU.

The code generator's float32 modules (heyoka's ``taylor_adaptive_batch`` with
``fp_type=numpy.float32``) are built for the host, both kernel forms, and compared bit
for bit with the oracle's float gpu-arithmetic step: every Taylor
coefficient and the stepped state.  The systems cover every operation and
operand kind (the float elementary functions included)."""

import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from hyk import _lib
from hyk.decompose import taylor_decompose

from test_team_codegen import CASES

pf = ctypes.POINTER(ctypes.c_float)


def _host(libhyk, sys_, order, team):
    d, keep = taylor_decompose(sys_).as_c()
    cfg = _lib.hyk_config_t(0, 0, _lib.HYK_CFG_FLOAT32, team)
    buf = ctypes.create_string_buffer(1 << 24)
    rc = libhyk.hyk_codegen_check(ctypes.byref(d), order, ctypes.byref(cfg), 3, buf, len(buf), None, None)
    assert rc == 0, libhyk.hyk_last_error()
    src = buf.value.decode()
    assert "typedef float hyk_real;" in src and "#define HYK_F32 1" in src
    tmp = tempfile.mkdtemp()
    cpp, so = os.path.join(tmp, "t.cpp"), os.path.join(tmp, "t.so")
    with open(cpp, "w") as f:
        f.write(src)
    subprocess.run(["g++", "-O1", "-ffp-contract=off", "-shared", "-fPIC", cpp, "-o", so], check=True)
    return ctypes.CDLL(so)


@pytest.mark.parametrize("form", ["team", "lane"])
@pytest.mark.parametrize("name", list(CASES))
def test_float_recurrences_bitwise_vs_oracle(libhyk, oracle, name, form):
    sys_, st, pars, order = CASES[name]()
    order = min(order, 10)  # float32 orders are about 9 (tolerance 2^-23)
    st = st.astype(np.float32).astype(np.float64)
    pars = None if pars is None else pars.astype(np.float32).astype(np.float64)
    H = _host(libhyk, sys_, order, team=2 if form == "team" else 1)
    o = oracle.Oracle(sys_, st, pars=pars, order=order, prec=2, mode=1, time=np.full(st.shape[1], 0.25))
    _, h = o.step()
    S = np.zeros(H.hyk_host_nslot(), dtype=np.float32)
    n_eq = st.shape[0]
    for lane in range(st.shape[1]):
        x0 = np.ascontiguousarray(st[:, lane], dtype=np.float32)
        p = np.ascontiguousarray(pars[:, lane] if pars is not None else np.zeros(1), dtype=np.float32)
        x1 = np.zeros(len(x0), dtype=np.float32)
        assert np.float32(h[lane]) == h[lane]
        H.hyk_host_step(S.ctypes.data_as(pf), x0.ctypes.data_as(pf), p.ctypes.data_as(pf), ctypes.c_float(0.25),
                        ctypes.c_float(h[lane]), x1.ctypes.data_as(pf))
        assert np.array_equal(x1.astype(np.float64), o.state[:, lane]), (name, lane)
        tc = np.zeros(n_eq * (order + 1), dtype=np.float32)
        H.hyk_host_tc(S.ctypes.data_as(pf), x0.ctypes.data_as(pf), p.ctypes.data_as(pf), ctypes.c_float(0.25),
                      tc.ctypes.data_as(pf))
        assert np.array_equal(tc.reshape(n_eq, order + 1).astype(np.float64), o.tc[:, :, lane]), (name, lane)


def test_float_step_close_to_double(oracle):
    """The float step follows the double one to single-precision accuracy."""
    sys_, st, pars, order = CASES["pendulum"]()
    st = st.astype(np.float32).astype(np.float64)
    of = oracle.Oracle(sys_, st, order=9, prec=2, mode=1)
    od = oracle.Oracle(sys_, st, order=9, prec=0, mode=1)
    _, hf = of.step()
    _, hd = od.step(max_delta_t=hf)
    assert np.allclose(of.state, od.state, rtol=0, atol=5e-6)


def test_float_module_rejects_pin_adjoint(libhyk):
    """Single precision has no pin arithmetic and no adjoint; the module
    constructor refuses them before it looks for a device."""
    import hyk

    x, v = hyk.make_vars("x", "v")
    d, keep = taylor_decompose([(x, v), (v, -hyk.sin(x))]).as_c()
    m = ctypes.c_void_p()
    for dec, extra in ((d, _lib.HYK_CFG_PIN_ARITH), (d, _lib.HYK_CFG_ADJOINT)):
        cfg = _lib.hyk_config_t(0, 0, _lib.HYK_CFG_FLOAT32 | extra, 0)
        rc = libhyk.hyk_module_create(ctypes.byref(dec), 9, ctypes.byref(cfg), 0, ctypes.byref(m))
        assert rc == _lib.HYK_ERR_UNSUPPORTED and b"single precision" in libhyk.hyk_last_error()


def test_float32_integrator_argument_checks():
    """Python-side checks of the float32 integrator that run before any device
    is touched: unsupported floating-point types."""
    import hyk

    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -hyk.sin(x))]
    with pytest.raises(TypeError, match="not recognized/supported"):
        hyk.taylor_adaptive_batch(sys_, [[0.1], [0.2]], fp_type=np.float16)
    with pytest.raises(TypeError, match="not recognized/supported"):
        hyk.t_event_batch(x, fp_type=np.float16)
    assert repr(hyk.t_event_batch(x, fp_type=np.float32)).startswith("C++ datatype: float")
