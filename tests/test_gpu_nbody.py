"""GPU parity for a system too large for shared memory: the outer-solar-system
6-body problem (Sun plus five bodies, 36 state variables, order 19 at
tol=1e-15).  Its Taylor coefficients do not fit 32 lanes of shared memory, so
the module keeps them in a global buffer; the arithmetic is unchanged and the
results stay bit-identical to the oracle.  The workload is the reference's
batch propagate_grid (heyoka/expose_batch_integrators.cpp:315-392) over a
per-lane grid of 100 points ending at per-lane times drawn log-uniformly.
"""

import numpy as np
import pytest
import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu


def _case(n, t_scale, seed=21):
    st, t_end = W.oss_ics(n, seed=seed)
    t_end = t_end * t_scale
    grid = np.linspace(0.0, 1.0, 100).reshape(-1, 1) * t_end.reshape(1, -1)
    return st, grid


def test_oss_form_choice(libhyk):
    # Automatic choice: the team form (one trajectory per team of threads,
    # coefficients in shared memory).  The lane form of this system keeps its
    # coefficients in global memory.
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), W.oss_ics(8)[0], tol=1e-15)
    info = ta.module_info
    assert info["n_eq"] == 36 and info["team_size"] > 1 and info["smem_per_lane"] > 0
    lane = hyk.taylor_adaptive_batch(W.oss_sys(), W.oss_ics(8)[0], tol=1e-15, team_size=1)
    assert lane.module_info["team_size"] == 1 and lane.module_info["smem_per_lane"] == 0


def test_oss_global_jets_lane_form_bitwise(oracle):
    st, grid = _case(24, 0.05, seed=24)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, team_size=1)
    _, out = ta.propagate_grid(grid)
    o = oracle.Oracle(W.oss_sys(), st, order=ta.order, mode=1)
    r = o.propagate_grid(grid)
    assert np.array_equal(out, r["grid"])


@pytest.mark.parametrize("mode", ["persistent", "plain"])
def test_oss_grid_bitwise(oracle, mode):
    st, grid = _case(48, 0.05)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15, prop_mode=mode)
    assert ta.order == 19
    _, out = ta.propagate_grid(grid)
    o = oracle.Oracle(W.oss_sys(), st, order=ta.order, mode=1)
    r = o.propagate_grid(grid)
    assert np.array_equal(out, r["grid"])
    assert np.array_equal(np.asarray(ta.state), o.state)
    g = {k: v.cpu().numpy() for k, v in ta.propagate_res_tensors.items()}
    assert np.array_equal(g["n_steps"], r["n_steps"].astype(np.int64))
    assert np.array_equal(g["min_h"], r["min_h"]) and np.array_equal(g["max_h"], r["max_h"])


def test_oss_more_lanes_than_threads(oracle):
    # More lanes than the fixed grid has threads: every thread walks several
    # lanes with the same coefficient slots; spot-check a subset bitwise.
    n = 40000
    st, grid = _case(n, 0.002, seed=22)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15)
    _, out = ta.propagate_grid(grid)
    pick = np.array([0, 1, 19455, 19456, 19457, 38911, 38912, n - 1])
    o = oracle.Oracle(W.oss_sys(), st[:, pick], order=ta.order, mode=1)
    r = o.propagate_grid(grid[:, pick])
    assert np.array_equal(out[:, :, pick], r["grid"])


def test_oss_energy_conserved():
    st, grid = _case(256, 0.2, seed=23)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15)
    e0 = W.oss_energy(st)
    ta.propagate_grid(grid)
    e1 = W.oss_energy(np.asarray(ta.state))
    assert np.all(np.isfinite(e1))
    assert np.max(np.abs((e1 - e0) / e0)) < 1e-11
