"""The multi-GPU ensemble's host logic on the CPU: iteration ranges per
device, the generator's iteration offsets, one replica per distinct device
and the results in iteration order (the device propagation replaced by a
recorder)."""

import threading

import pytest

from hyk import ensemble
from hyk.integrator import taylor_adaptive_batch


def _fake(dev):
    t = object.__new__(taylor_adaptive_batch)
    t.__dict__["_dev"] = dev
    return t


def test_devices_partition_order_and_offsets(monkeypatch):
    calls = []
    lock = threading.Lock()

    def fake_ensemble(tp, ta, arg, n, gen, **kw):
        assert "devices" not in kw
        out = [(ta._dev, gen(None, i)) for i in range(n)]
        with lock:
            calls.append((ta._dev, n))
        return out

    made = []

    def fake_replica(self, device):
        made.append(device)
        return _fake(int(str(device).split(":")[-1]))

    monkeypatch.setattr(ensemble, "_ensemble", fake_ensemble)
    monkeypatch.setattr(taylor_adaptive_batch, "_replica", fake_replica)
    tmpl = _fake(0)
    res = ensemble._ensemble_devices("until", tmpl, 1.0, 10, lambda c, i: i, ["cuda:0", "cuda:1", "cuda:1"], {})
    assert [r[1] for r in res] == list(range(10))  # iteration order, every offset once
    assert [r[0] for r in res] == [0] * 3 + [1] * 7  # ranges [0,3) [3,6) [6,10): device 0, 1, 1
    assert sorted(calls) == [(0, 3), (1, 3), (1, 4)]
    assert made == [1]  # one replica per distinct device; device 0 uses the template
    assert ensemble._ensemble_devices("until", tmpl, 1.0, 0, lambda c, i: i, ["cuda:0"], {}) == []


def test_devices_validation(monkeypatch):
    tmpl = _fake(0)
    with pytest.raises(ValueError):
        ensemble._ensemble_devices("until", tmpl, 1.0, 4, lambda c, i: c, [], {})
    with pytest.raises(TypeError):  # the single-device path's own argument errors
        ensemble._ensemble_devices("until", tmpl, [1.0, 2.0], 4, lambda c, i: c, ["cuda:0"], {})
    with pytest.raises(ValueError):
        ensemble._ensemble_devices("until", tmpl, 1.0, 4, lambda c, i: c, ["cpu"], {})
