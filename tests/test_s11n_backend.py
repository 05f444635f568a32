"""The serialization backend switch (heyoka/test.py s11n_backend_test_case,
heyoka/__init__.py:180-238) and event callbacks pickled with each backend."""

import pickle

import pytest

import hyk


def test_backend_switch():
    cp = pytest.importorskip("cloudpickle")
    assert hyk.get_serialization_backend() is cp
    hyk.set_serialization_backend("pickle")
    assert hyk.get_serialization_backend() is pickle
    hyk.set_serialization_backend("cloudpickle")
    assert hyk.get_serialization_backend() is cp
    with pytest.raises(TypeError, match="The serialization backend must be specified as a string"):
        hyk.set_serialization_backend(1)
    with pytest.raises(ValueError, match="The serialization backend 'pippo' is not valid. The valid backends are:"):
        hyk.set_serialization_backend("pippo")
    assert hyk.get_serialization_backend() is cp


class _Cb:
    def __init__(self):
        self.n = 0

    def __call__(self, ta, t, d_sgn, bidx):
        self.n += 1


def test_event_callback_pickled_with_active_backend():
    x, v = hyk.make_vars("x", "v")
    old = hyk.get_serialization_backend()
    try:
        for name in ("pickle", "cloudpickle"):
            if name == "cloudpickle":
                pytest.importorskip("cloudpickle")
            hyk.set_serialization_backend(name)
            cb = _Cb()
            cb.n = 7
            ev = hyk.nt_event_batch(v * v - 1e-10, cb)
            ev2 = pickle.loads(pickle.dumps(ev))
            assert isinstance(ev2.callback, _Cb) and ev2.callback.n == 7
            assert ev2.expression == ev.expression
        # a local function needs cloudpickle; the standard pickle refuses it
        pytest.importorskip("cloudpickle")

        def local_cb(ta, t, d_sgn, bidx):
            pass

        hyk.set_serialization_backend("cloudpickle")
        ev = pickle.loads(pickle.dumps(hyk.nt_event_batch(v * v - 1e-10, local_cb)))
        assert callable(ev.callback)
        hyk.set_serialization_backend("pickle")
        with pytest.raises((pickle.PicklingError, AttributeError)):
            pickle.dumps(hyk.nt_event_batch(v * v - 1e-10, local_cb))
    finally:
        hyk.set_serialization_backend(hyk.s11n._backend_inv[id(old)])
