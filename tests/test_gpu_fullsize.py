"""Parity at the benchmark configurations' full sizes.

The oracle cannot integrate 2^20 orbits in seconds, so at full size the
checks are the size-independent ones: every lane reaches its final time
exactly with the time-limit outcome, the first integrals of each system
(energy and angular momentum of the Kepler orbits, total energy of the
6-body problem, the CR3BP Hamiltonian in the rotating frame, the pendulum's
energy) are conserved to the integrator's accuracy, and a seeded sample of
lanes out of each full batch is bit-for-bit identical, state and step count,
to the oracle's gpu arithmetic on the same lanes (a lane's arithmetic does
not depend on the batch around it)."""

import numpy as np
import pytest
import torch

import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu


def _sample(n, k, seed):
    return np.sort(np.random.default_rng(seed).choice(n, k, replace=False))


def _kepler_invariants(st):
    r, v = st[0:3], st[3:6]
    e = 0.5 * np.sum(v * v, axis=0) - 1.0 / np.sqrt(np.sum(r * r, axis=0))
    h = np.cross(r.T, v.T).T
    return e, h


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def test_kepler_2p20_full(oracle):
    """2^20 Kepler orbits, tol 1e-15 (order 19), t = 0..200."""
    n = 1 << 20
    st = W.kepler_ics(n, seed=1)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    ta.propagate_until(200.0)
    res = ta.propagate_res_tensors
    assert bool((res["outcome"] == int(hyk.taylor_outcome.time_limit)).all())
    assert np.all(ta.time == 200.0)
    fin = np.asarray(ta.state)
    e0, h0 = _kepler_invariants(st)
    e1, h1 = _kepler_invariants(fin)
    de = _rel(e1, e0)
    dh = np.linalg.norm(h1 - h0, axis=0) / np.linalg.norm(h0, axis=0)
    print("kepler 2^20: max rel energy drift %.3g, max rel |h| drift %.3g, steps %d" % (
        de.max(), dh.max(), int(res["n_steps"].sum())))
    assert de.max() < 1e-12 and dh.max() < 1e-12
    pick = _sample(n, 256, 11)
    o = oracle.Oracle(W.kepler_sys(), st[:, pick], order=ta.order, mode=1)
    o.propagate_until(200.0)
    assert np.array_equal(fin[:, pick], o.state)


def test_oss_65536_grid_full(oracle):
    """65536 outer-solar-system members, tol 1e-15, end times log-uniform in
    [1e3, 1e5] days, propagate_grid over 100 points per member."""
    n = 65536
    st, t_end = W.oss_ics(n, seed=2)
    grid = np.linspace(0.0, 1.0, 100).reshape(-1, 1) * t_end.reshape(1, -1)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15)
    out = ta.propagate_grid_tensor(torch.tensor(grid, device="cuda"))
    assert bool(torch.isfinite(out).all())
    assert np.array_equal(ta.time, t_end)
    fin = np.asarray(ta.state)
    assert torch.allclose(out[-1], ta.state.as_subclass(torch.Tensor), rtol=1e-13, atol=0)
    de = _rel(W.oss_energy(fin), W.oss_energy(st))
    print("oss 65536: max rel energy drift %.3g" % de.max())
    assert de.max() < 1e-12
    pick = _sample(n, 12, 12)
    o = oracle.Oracle(W.oss_sys(), st[:, pick], order=ta.order, mode=1)
    r = o.propagate_grid(grid[:, pick])
    assert np.array_equal(out[:, :, pick].cpu().numpy(), r["grid"])
    assert np.array_equal(fin[:, pick], o.state)


def _cr3bp_h(st, mu):
    x, y, z, px, py, pz = st
    r1 = np.sqrt((x - mu) ** 2 + y * y + z * z)
    r2 = np.sqrt((x - mu + 1.0) ** 2 + y * y + z * z)
    return 0.5 * (px * px + py * py + pz * pz) + y * px - x * py - (1.0 - mu) / r1 - mu / r2


def test_cr3bp_65536_full(oracle):
    """65536 CR3BP trajectories near L4, mu per lane, tol 1e-15, t = 0..50."""
    n = 65536
    st, mu = W.cr3bp_ics(n, seed=3)
    ta = hyk.taylor_adaptive_batch(W.cr3bp_sys(), st, pars=mu, tol=1e-15)
    ta.propagate_until(50.0)
    assert bool((ta.propagate_res_tensors["outcome"] == int(hyk.taylor_outcome.time_limit)).all())
    assert np.all(ta.time == 50.0)
    fin = np.asarray(ta.state)
    dh = _rel(_cr3bp_h(fin, mu[0]), _cr3bp_h(st, mu[0]))
    print("cr3bp 65536: max rel Hamiltonian drift %.3g" % dh.max())
    assert dh.max() < 1e-12
    pick = _sample(n, 256, 13)
    o = oracle.Oracle(W.cr3bp_sys(), st[:, pick], pars=mu[:, pick], order=ta.order, mode=1)
    o.propagate_until(50.0)
    assert np.array_equal(fin[:, pick], o.state)


def test_pendulum_ensemble_4096_full(oracle):
    """4096 pendulum trajectories as 1024 ensemble iterations of batch 4,
    tol 2.2e-16 (order 20), t = 0..100."""
    rng = np.random.default_rng(0)
    x0 = rng.uniform(-1.5, 1.5, 4096)
    v0 = rng.uniform(-0.5, 0.5, 4096)
    st = np.stack([x0, v0])
    ta = hyk.taylor_adaptive_batch(W.pendulum_sys(), st[:, :4], tol=2.2e-16)

    def gen(t, i):
        t.state[:] = st[:, 4 * i: 4 * i + 4]
        return t

    res = hyk.ensemble_propagate_until(ta, 100.0, 1024, gen)
    fin = np.concatenate([np.asarray(r[0].state) for r in res], axis=1)
    assert all(np.all(r[0].time == 100.0) for r in res)
    en = lambda s: 0.5 * s[1] ** 2 - 9.8 * np.cos(s[0])  # noqa: E731
    de = np.abs(en(fin) - en(st)) / np.abs(en(st))
    print("pendulum 4096: max rel energy drift %.3g" % de.max())
    assert de.max() < 1e-12
    pick = _sample(4096, 64, 14)
    o = oracle.Oracle(W.pendulum_sys(), st[:, pick], order=ta.order, mode=1)
    o.propagate_until(100.0)
    assert np.array_equal(fin[:, pick], o.state)
