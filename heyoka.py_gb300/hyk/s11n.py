"""The serialization backend for the Python objects held by integrators
(event callbacks), as in the reference (heyoka/__init__.py:180-238,
set_serialization_backend / get_serialization_backend; used when pickling
events, heyoka/taylor_expose_events.cpp:142-163).  The default is cloudpickle
when it is installed, else the standard pickle module."""

from __future__ import annotations

import pickle
import threading


def _make_maps():
    ret = {"pickle": pickle}
    try:
        import cloudpickle

        ret["cloudpickle"] = cloudpickle
    except ImportError:
        pass
    try:
        import dill

        ret["dill"] = dill
    except ImportError:
        pass
    return ret, {id(m): n for n, m in ret.items()}


_backend_map, _backend_inv = _make_maps()
_backend = _backend_map.get("cloudpickle", pickle)
_mutex = threading.Lock()


def set_serialization_backend(name):
    global _backend
    if not isinstance(name, str):
        raise TypeError("The serialization backend must be specified as a string, but an object of type {} was "
                        "provided instead".format(type(name)))
    if name not in _backend_map:
        raise ValueError("The serialization backend '{}' is not valid. The valid backends are: {}".format(
            name, list(_backend_map.keys())))
    with _mutex:
        _backend = _backend_map[name]


def get_serialization_backend():
    with _mutex:
        return _backend


def dumps(obj):
    """(backend name, bytes) of obj with the active backend."""
    be = get_serialization_backend()
    data = be.dumps(obj)
    if not isinstance(data, bytes):
        raise TypeError("The serialization backend's dumps() function did not return a bytes object")
    return (_backend_inv[id(be)], data)


def loads(blob):
    name, data = blob
    return _backend_map.get(name, pickle).loads(data)


__all__ = ["get_serialization_backend", "set_serialization_backend"]
