"""Compiled CPU batch stepper (TEST INFRASTRUCTURE: the timed CPU baseline).

The reference's timed path is heyoka's LLVM-compiled batch stepper behind
``taylor_adaptive_batch.propagate_until`` (heyoka/expose_batch_integrators.cpp:279-314),
fanned out over host threads by ``ensemble_propagate_until``
(heyoka/_ensemble_impl.py:23-68).  It cannot be built here; this module stands
in for it: the system's recurrences are generated as straight-line C++ in the
reference's arithmetic (libhyk's code generator, ``hyk_codegen_check`` with
verbose 4), compiled with ``g++ -O3`` together with ``hyk_cpu_batch.cpp`` (the
oracle's batch propagate loop over vectors of ``batch`` lanes), and run over
all host threads.  Its results are the oracle's "pin" arithmetic
(``tests/test_cpu_batch.py`` checks them against ``pyoracle``).

Only bench.py's CPU-baseline leg and the tests use this module.
"""

from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if os.path.join(ROOT, "heyoka.py_gb300") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "heyoka.py_gb300"))
OUT_DIR = os.path.join(HERE, "_build")

_CACHE = {}
_PEAK = None

FLAGS = ["-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wno-psabi", "-fPIC", "-shared"]


def _generate(dec, order: int) -> str:
    from hyk import _lib

    L = _lib.load()
    cdec, keep = dec.as_c()
    buf = ctypes.create_string_buffer(1 << 25)
    rc = L.hyk_codegen_check(ctypes.byref(cdec), int(order), None, 4, buf, len(buf), None, None)
    if rc != 0:
        raise RuntimeError("hyk_codegen_check: " + L.hyk_last_error().decode())
    del keep
    return buf.value.decode()


def stepper(sys_or_dec, order: int, batch: int = 8):
    """The compiled stepper of a system (cached per decomposition, order and batch width)."""
    from hyk.decompose import Decomposition, taylor_decompose

    dec = sys_or_dec if isinstance(sys_or_dec, Decomposition) else taylor_decompose(sys_or_dec)
    key = (dec.digest(), int(order), int(batch))
    if key in _CACHE:
        return _CACHE[key]
    src = _generate(dec, order)
    drv = os.path.join(HERE, "hyk_cpu_batch.cpp")
    tag = hashlib.sha1((src + open(drv).read() + " ".join(FLAGS) + str(batch)).encode()).hexdigest()[:16]
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = os.path.join(OUT_DIR, "cpu_jets_{}.inc".format(tag))
    so = os.path.join(OUT_DIR, "libhyk_cpu_{}.so".format(tag))
    if not os.path.exists(so):
        with open(inc, "w") as f:
            f.write(src)
        tmp = so + ".{}.tmp".format(os.getpid())
        subprocess.run(["g++"] + FLAGS + ["-DHYK_B={}".format(int(batch)), "-DHYK_JETS_INC=" + inc, drv, "-o", tmp],
                       check=True)
        os.replace(tmp, so)
    L = ctypes.CDLL(so)
    P = ctypes.POINTER
    L.hyk_cpu_until.restype = ctypes.c_int
    L.hyk_cpu_until.argtypes = [ctypes.c_uint64, ctypes.c_uint64, P(ctypes.c_double), P(ctypes.c_double), ctypes.c_double,
                                P(ctypes.c_double), ctypes.c_int, P(ctypes.c_double), P(ctypes.c_int64),
                                P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_uint64)]
    _CACHE[key] = L
    return L


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def ensemble_until(sys_or_dec, state, pars, t0: float, tf, order: int, batch: int = 8, n_threads: int = 0):
    """propagate_until(tf) of every lane of ``state`` ((n_eq, n) array) from time t0; ``tf`` a scalar or one
    end time per lane."""
    L = stepper(sys_or_dec, order, batch)
    st = np.ascontiguousarray(state, dtype=np.float64)
    n = st.shape[1]
    pa = np.ascontiguousarray(pars if pars is not None else np.zeros((1, n)), dtype=np.float64)
    out = np.empty_like(st)
    oc = np.empty(n, dtype=np.int64)
    mn, mx = np.empty(n), np.empty(n)
    ns = np.empty(n, dtype=np.uint64)
    tfa = np.ascontiguousarray(np.broadcast_to(np.asarray(tf, dtype=np.float64), (n,)))
    used = L.hyk_cpu_until(n, n, _p(st), _p(pa), float(t0), _p(tfa), int(n_threads), _p(out), _p(oc, ctypes.c_int64),
                           _p(mn), _p(mx), _p(ns, ctypes.c_uint64))
    return {"state": out, "outcome": oc, "min_h": mn, "max_h": mx, "n_steps": ns, "threads": used}


def fp64_peak(n_threads: int = 0, seconds: float = 1.0):
    """FP64 FMA flop/s of the host cores (hyk_cpu_peak.c), calibrated to about ``seconds``."""
    global _PEAK
    if _PEAK is None:
        src = os.path.join(HERE, "hyk_cpu_peak.c")
        so = os.path.join(OUT_DIR, "libhyk_cpu_peak.so")
        if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
            os.makedirs(OUT_DIR, exist_ok=True)
            tmp = so + ".{}.tmp".format(os.getpid())
            subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=fast", "-fPIC", "-shared", src, "-o", tmp], check=True)
            os.replace(tmp, so)
        _PEAK = ctypes.CDLL(so)
        _PEAK.hyk_cpu_fma_peak.restype = ctypes.c_double
        _PEAK.hyk_cpu_fma_peak.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]
    secs, chk = ctypes.c_double(), ctypes.c_double()
    iters = 1 << 16
    while True:
        f = _PEAK.hyk_cpu_fma_peak(int(n_threads), iters, ctypes.byref(secs), ctypes.byref(chk))
        if secs.value >= 0.1 * seconds or iters > (1 << 40):
            break
        iters *= 4
    iters = max(1, int(iters * seconds / max(secs.value, 1e-9)))
    best = 0.0
    for _ in range(2):
        best = max(best, _PEAK.hyk_cpu_fma_peak(int(n_threads), iters, ctypes.byref(secs), ctypes.byref(chk)))
    return best
