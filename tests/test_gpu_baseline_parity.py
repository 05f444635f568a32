"""Parity with the reference's arithmetic at the benchmark configurations.

The GPU's default path (fused multiply-adds, reciprocal multiplications, this
project's elementary functions) is compared with the oracle in "pin"
arithmetic, the arithmetic that reproduces the reference's recorded outputs
(no fused multiply-adds, true divisions, the C library's functions), on
seeded subsamples of the benchmark ensembles:

* Kepler: 1024 of the 2^20 orbits of the headline benchmark, tol 1e-15
  (order 19), propagated to t = 20, 50 and 200;
* CR3BP near L4: 1024 of the 65536 trajectories, t = 50;
* the outer-solar-system 6-body ensemble: 64 of the 65536 members,
  propagate_grid at 100 points up to each member's end time.

Criteria: identical step counts on at least 99 % of trajectories, and a
per-trajectory final-state relative error (2-norm of the difference over
the 2-norm of the state) of at most 1e-12, on CR3BP, on the 6-body
ensemble and on Kepler up to t = 20.  Beyond that horizon the Kepler orbits
(eccentricities up to 0.6, up to 90 revolutions) amplify rounding: the
reference arithmetic itself is farther than 1e-12 from the binary128
solution on some orbits (2.3e-12 at t = 50, 1.3e-11 at t = 200), so two
arithmetics that are not bit-identical cannot agree to 1e-12 there.  At
t = 50 and t = 200 the test therefore measures both against the binary128
states of tests/golden/kepler_t200_quad_1024.npz and requires the GPU's
error distribution to be no worse than the reference arithmetic's: median and
90th percentile within 25 %, 99th percentile within 50 %.  The maximum over
1024 orbits of this heavy-tailed error is a lottery: the orbits that amplify
rounding most are hit hardest by different orbits' rounding in the two
arithmetics (per orbit, log2 of the ratio of the two errors has mean -0.03 at
t = 200), so the maximum is only required within 3x.
"""

import os

import numpy as np
import pytest
import torch

import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kepler_t200_quad_1024.npz")


@pytest.fixture(scope="module", autouse=True)
def _built(libhyk):
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    yield


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)


def test_kepler_1024_orbits_to_t200(oracle):
    fx = np.load(GOLDEN)
    st = np.ascontiguousarray(W.kepler_ics(1 << 20, seed=1)[:, fx["idx"]])
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    assert ta.order == 19
    ref = oracle.Oracle(W.kepler_sys(), st, order=19, mode=0)
    report = {}
    for t in (20.0, 50.0, 200.0):
        ta.propagate_until(t)
        r = ref.propagate_until(t)
        g = np.asarray(ta.state)
        ns = ta.propagate_res_tensors["n_steps"].cpu().numpy()
        assert np.all(ta.propagate_res_tensors["outcome"].cpu().numpy() == int(hyk.taylor_outcome.time_limit))
        agree = float(np.mean(ns == r["n_steps"].astype(np.int64)))
        assert agree >= 0.99, (t, agree)
        e = rel_err(g, ref.state)
        report[t] = (e.max(), agree)
        if t == 20.0:
            assert e.max() <= 1e-12, e.max()
            continue
        q = fx["state_t{:g}".format(t)]
        eg, er = rel_err(g, q), rel_err(ref.state, q)
        # the GPU is as accurate as the reference arithmetic against the binary128 solution
        assert np.median(eg) <= 1.25 * np.median(er), t
        assert np.quantile(eg, 0.9) <= 1.25 * np.quantile(er, 0.9), t
        assert np.quantile(eg, 0.99) <= 1.5 * np.quantile(er, 0.99), t
        assert eg.max() <= 3.0 * er.max(), (t, eg.max(), er.max())
    print("kepler 1024: (max rel err vs reference arithmetic, step agreement)", report)


def test_cr3bp_1024_trajectories_to_t50(oracle):
    st, pars = W.cr3bp_ics(1 << 16, seed=3)
    idx = np.sort(np.random.default_rng(123).choice(1 << 16, 1024, replace=False))
    st, pars = np.ascontiguousarray(st[:, idx]), np.ascontiguousarray(pars[:, idx])
    ta = hyk.taylor_adaptive_batch(W.cr3bp_sys(), st, pars=pars, tol=1e-15)
    ta.propagate_until(50.0)
    ref = oracle.Oracle(W.cr3bp_sys(), st, pars=pars, order=ta.order, mode=0)
    r = ref.propagate_until(50.0)
    e = rel_err(np.asarray(ta.state), ref.state)
    assert e.max() <= 1e-12, e.max()
    ns = ta.propagate_res_tensors["n_steps"].cpu().numpy()
    assert np.mean(ns == r["n_steps"].astype(np.int64)) >= 0.99


def test_oss_64_members_grid_to_t_end(oracle):
    st, t_end = W.oss_ics(1 << 16, seed=2)
    idx = np.sort(np.random.default_rng(123).choice(1 << 16, 64, replace=False))
    st, t_end = np.ascontiguousarray(st[:, idx]), t_end[idx]
    grid = np.linspace(0.0, 1.0, 100).reshape(-1, 1) * t_end.reshape(1, -1)
    ta = hyk.taylor_adaptive_batch(W.oss_sys(), st, tol=1e-15)
    _, out = ta.propagate_grid(grid)
    ref = oracle.Oracle(W.oss_sys(), st, order=ta.order, mode=0)
    r = ref.propagate_grid(grid)
    e = rel_err(np.asarray(ta.state), ref.state)
    assert e.max() <= 1e-12, e.max()
    # every grid row, as a state
    eg = np.linalg.norm(out - r["grid"], axis=1) / np.linalg.norm(r["grid"], axis=1)
    assert eg.max() <= 1e-12, eg.max()
    ns = ta.propagate_res_tensors["n_steps"].cpu().numpy()
    assert np.mean(ns == r["n_steps"].astype(np.int64)) >= 0.99
