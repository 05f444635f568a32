"""The kernel-configuration autotuner: cache and helpers on the CPU, the
measurement and the integrator option on the GPU."""

import numpy as np
import pytest
import torch

import hyk
from hyk import autotune
from hyk import workloads as W
from hyk.decompose import taylor_decompose


def test_cache_roundtrip_and_keys(tmp_path, monkeypatch):
    monkeypatch.setenv("HYK_CACHE_DIR", str(tmp_path))
    dec = taylor_decompose(W.kepler_sys())
    k64 = autotune.cache_key(dec, 19, "GPU", False, False)
    k32 = autotune.cache_key(dec, 9, "GPU", True, False)
    kha = autotune.cache_key(dec, 19, "GPU", False, True)
    assert len({k64, k32, kha}) == 3 and dec.digest() in k64
    assert autotune._load_cache() == {}
    autotune._store_cache(k64, {"best": {"team_size": 1, "global_jets": False, "block_lanes": 0}, "rate": 1.0})
    autotune._store_cache(k32, {"best": {"team_size": 2, "global_jets": False, "block_lanes": 0}, "rate": 2.0})
    data = autotune._load_cache()
    assert data[k64]["best"]["team_size"] == 1 and data[k32]["best"]["team_size"] == 2
    assert (tmp_path / "autotune.json").exists()


def test_replicate():
    a = np.arange(6.0).reshape(2, 3)
    r = autotune._replicate(a, 7)
    assert r.shape == (2, 7) and r.flags.c_contiguous
    assert np.array_equal(r[:, :3], a) and np.array_equal(r[:, 3:6], a) and np.array_equal(r[:, 6], a[:, 0])
    assert autotune._replicate(None, 5) is None


@pytest.mark.gpu
def test_tune_measures_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("HYK_CACHE_DIR", str(tmp_path))
    st = W.pendulum_ics(64, seed=3)
    r = autotune.tune(W.pendulum_sys(), st, steps=8, lanes=8192,
                      candidates=((1, False, 0), (1, True, 0), (2, False, 0), (4, False, 0)))
    assert not r["cached"] and r["rate"] > 0
    measured = [t for t in r["trials"] if "trajectory_steps_per_s" in t]
    assert len(measured) >= 3
    # the constructor's choice is kept unless another is faster by the margin
    assert r["rate"] * autotune.MARGIN >= max(t["trajectory_steps_per_s"] for t in measured)
    assert r["rate_grid"] * autotune.MARGIN >= max(t["grid_trajectory_steps_per_s"] for t in measured)
    assert "best_grid" in r
    r2 = autotune.tune(W.pendulum_sys(), st, steps=8, lanes=8192)
    assert r2["cached"] and r2["best"] == r["best"]
    # an integrator built with autotune=True uses the cached choice, and every
    # configuration gives the same bits
    a = hyk.taylor_adaptive_batch(W.pendulum_sys(), st, autotune=True)
    assert a._autotune["cached"] and a._mod_opts["team_size"] == r["best"]["team_size"]
    b = hyk.taylor_adaptive_batch(W.pendulum_sys(), st)
    a.propagate_until(10.0)
    b.propagate_until(10.0)
    assert torch.equal(a.state, b.state) and a.propagate_res == b.propagate_res


@pytest.mark.gpu
def test_tune_call_on_the_callers_workload():
    st = W.kepler_ics(8192, seed=4)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    ref = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    s0 = ta.state.clone()
    r = autotune.tune_call(ta, lambda t: t.propagate_until(2.0),
                           candidates=((0, False, 0), (1, True, 0), (2, False, 0)))
    timed = [t for t in r["trials"] if "seconds" in t]
    assert len(timed) >= 2 and r["seconds"] == min(t["seconds"] for t in timed)
    assert torch.equal(ta.state, s0) and np.all(ta.time == 0.0)  # inputs restored
    ta.propagate_until(2.0)
    ref.propagate_until(2.0)
    assert torch.equal(ta.state, ref.state) and ta.propagate_res == ref.propagate_res
    assert ta._mod_opts["team_size"] == r["best"]["team_size"]


@pytest.mark.gpu
def test_modules_are_freed():
    from hyk import core

    st = W.pendulum_ics(8, seed=1)
    ta = hyk.taylor_adaptive_batch(W.pendulum_sys(), st, team_size=2)
    m = ta._mod
    core.drop_modules()
    assert m.handle is not None  # still used by ta
    ta.propagate_until(1.0)
    del ta
    import gc

    gc.collect()
    assert m.handle is not None  # the test's own reference keeps it
    m.close()
    assert m.handle is None
