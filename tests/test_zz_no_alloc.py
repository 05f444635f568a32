"""hyk_propagate_noalloc: propagation for callers that cannot allocate.

Some callers of this library cannot call cudaMalloc (code running inside
another allocator's pool, a real-time loop that must not allocate, a host
integration without a CUDA allocator), so they cannot hand hyk_propagate the
small device workspace it keeps its lane-queue and finished-lane counters in.
hyk_propagate_noalloc takes no workspace: the counters live in a file-scope
device array inside libhyk.  This test calls it through the C ABI and checks
that it reproduces hyk_propagate's results exactly, on two calls in a row
(the second call reuses the array the first one left behind), in both the
persistent and the one-launch-per-step form.  It is collected last so that a
run stopping at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

from hyk import _lib, workloads as W
from hyk.core import get_module, lanes_struct, stream_handle
from hyk.decompose import order_from_tol, taylor_decompose

pytestmark = pytest.mark.gpu


def _arrays(n, dev):
    f = dict(device=dev)
    return {
        "rem_hi": torch.empty(n, dtype=torch.float64, **f),
        "rem_lo": torch.empty(n, dtype=torch.float64, **f),
        "outcome": torch.empty(n, dtype=torch.int64, **f),
        "min_h": torch.empty(n, dtype=torch.float64, **f),
        "max_h": torch.empty(n, dtype=torch.float64, **f),
        "n_steps": torch.empty(n, dtype=torch.int64, **f),
        "n_iter": torch.empty(n, dtype=torch.int64, **f),
        "last_h": torch.empty(n, dtype=torch.float64, **f),
        "status": torch.empty(n, dtype=torch.int32, **f),
    }


def _desc(tf, a):
    return _lib.hyk_prop_t(
        tf.data_ptr(), None, None, 0, None, 0, None, None, None, None, 0,
        a["rem_hi"].data_ptr(), a["rem_lo"].data_ptr(), a["outcome"].data_ptr(), a["min_h"].data_ptr(),
        a["max_h"].data_ptr(), a["n_steps"].data_ptr(), a["n_iter"].data_ptr(), None, a["last_h"].data_ptr(),
        None, a["status"].data_ptr(), None, 0, None, None, None, 0, 0,
    )


def _propagate(L, mod, st, tf, dev, noalloc, mode):
    """Propagate a copy of `st` from t = 0 to tf in two calls (to tf/2, then tf)."""
    n = st.shape[1]
    state = torch.tensor(st, dtype=torch.float64, device=dev)
    th = torch.zeros(n, dtype=torch.float64, device=dev)
    tl = torch.zeros(n, dtype=torch.float64, device=dev)
    lanes = lanes_struct(state, None, th, tl)
    s = stream_handle(dev.index)
    ws = torch.zeros(64, dtype=torch.int32, device=dev)
    results = []
    for target in (0.5 * tf, tf):
        t = torch.full((n,), target, dtype=torch.float64, device=dev)
        a = _arrays(n, dev)
        d = _desc(t, a)
        _lib.check(L.hyk_prop_init(mod.handle, lanes, d, s), "hyk_prop_init")
        if noalloc:
            rc = L.hyk_propagate_noalloc(mod.handle, lanes, d, mode, 16, None, s)
        else:
            rc = L.hyk_propagate(mod.handle, lanes, d, mode, ws.data_ptr(), 256, 16, None, s)
        _lib.check(rc, "propagate")
        torch.cuda.synchronize(dev)
        results.append((state.cpu().numpy().copy(), th.cpu().numpy().copy(), {k: v.cpu().numpy() for k, v in a.items()}))
    return results


@pytest.mark.parametrize("n", [300, 5000])
@pytest.mark.parametrize("mode", [_lib.HYK_MODE_PERSISTENT, _lib.HYK_MODE_PLAIN])
def test_noalloc_matches_workspace_entry_point(libhyk, mode, n):
    """With 300 lanes the plain form's lane list fits the no-allocation scratch
    (it steps the listed unfinished lanes); with 5000 it steps the lanes in
    place, as the 256-byte workspace of the other entry point makes it do."""
    assert torch.cuda.is_available(), "this test needs a CUDA device"
    dev = torch.device("cuda", 0)
    dec = taylor_decompose(W.kepler_sys())
    mod = get_module(dec, order_from_tol(1e-15), 0)
    assert int(libhyk.hyk_propagate_workspace_size(mod.handle, n, _lib.HYK_MODE_PLAIN)) == 256 + 8 * n
    assert int(libhyk.hyk_propagate_workspace_size(mod.handle, n, _lib.HYK_MODE_PERSISTENT)) == 256
    st = W.kepler_ics(n, seed=21)
    ref = _propagate(libhyk, mod, st, 6.0, dev, noalloc=False, mode=mode)
    got = _propagate(libhyk, mod, st, 6.0, dev, noalloc=True, mode=mode)
    for (s0, t0, a0), (s1, t1, a1) in zip(ref, got):
        # The integration is deterministic: the tolerance of the other parity tests (bit-identical) applies.
        assert np.array_equal(s0, s1) and np.array_equal(t0, t1)
        for k in ("n_steps", "n_iter", "min_h", "max_h", "outcome", "status"):
            assert np.array_equal(a0[k], a1[k]), k
        assert np.all(a1["n_steps"] > 0)


def test_noalloc_scratch_per_device(libhyk):
    """Every GPU that loads the library holds its own copy of the scratch
    array, and its address is looked up on that device.  With two GPUs, a
    call on device 1 after one on device 0 must still reproduce hyk_propagate
    on both (a device-0 address used on device 1 would not)."""
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two visible GPUs")
    dec = taylor_decompose(W.kepler_sys())
    st = W.kepler_ics(300, seed=22)
    for ordinal in (0, 1):
        dev = torch.device("cuda", ordinal)
        mod = get_module(dec, order_from_tol(1e-15), ordinal)
        for mode in (_lib.HYK_MODE_PERSISTENT, _lib.HYK_MODE_PLAIN):
            ref = _propagate(libhyk, mod, st, 6.0, dev, noalloc=False, mode=mode)
            got = _propagate(libhyk, mod, st, 6.0, dev, noalloc=True, mode=mode)
            for (s0, t0, a0), (s1, t1, a1) in zip(ref, got):
                assert np.array_equal(s0, s1) and np.array_equal(t0, t1)
                assert np.array_equal(a0["n_steps"], a1["n_steps"])
