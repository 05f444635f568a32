"""Every operation kind of the code generator on the GPU, bit for bit.

The benchmark systems (pendulum, Kepler, CR3BP, N-body) use only add, sub,
mul, neg, square, pow, sin and cos with variable, number and parameter
operands.  These systems add exp, log, sqrt, div, the time as an operand,
time-constant operations (numbers and parameters combined before the
recurrences) and an order-2 variational system, and run them through every
kernel form: the lane form with coefficients in shared memory, the lane form
with coefficients in global memory, and teams of 2 and 8 threads per
trajectory, each in the persistent and the one-launch-per-step propagation.
The GPU must equal the oracle's gpu arithmetic bit for bit: states, times,
step counts, min/max step sizes, and for one form the Taylor coefficients of
single steps and a dense-output grid."""

import numpy as np
import pytest
import torch

import hyk
import systems

pytestmark = pytest.mark.gpu


def _case(name, n=96):
    rng = np.random.default_rng({"mixed": 41, "consts": 42, "var2": 43}[name])
    if name == "mixed":
        st = np.vstack([rng.uniform(1.0, 1.3, n), rng.uniform(0.7, 0.9, n)])
        pars = np.vstack([rng.uniform(0.1, 0.3, n), rng.uniform(0.3, 0.6, n)])
        return systems.mixed(), st, pars, 1e-15, 0.4
    if name == "consts":
        st = np.vstack([rng.uniform(0.1, 0.3, n), rng.uniform(0.4, 0.6, n)])
        pars = np.vstack([rng.uniform(0.1, 0.3, n), rng.uniform(0.3, 0.6, n)])
        return systems.consts(), st, pars, 1e-15, 1.0
    return systems.var2().sys, systems.var2_state(n, rng), np.full((1, n), 0.4), 2.2e-16, 4.0


FORMS = {
    "lane_smem": dict(),
    "lane_gmem": dict(global_jets=True),
    "team2": dict(team_size=2),
    "team8": dict(team_size=8),
}


@pytest.fixture(scope="module", autouse=True)
def _built(libhyk):
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    yield


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("name", ["mixed", "consts", "var2"])
def test_ops_propagate_until_bitwise(oracle, name, form, mode):
    sys_, st, pars, tol, tf = _case(name)
    # uneven end times, so that lanes finish many launches apart
    tf = np.linspace(0.5 * tf, tf, st.shape[1])
    ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=tol, prop_mode=mode, **FORMS[form])
    info = ta.module_info
    if form.startswith("team"):
        assert info["team_size"] == FORMS[form]["team_size"]
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st, pars=pars, order=ta.order, mode=1)
    r = o.propagate_until(tf)
    g = {k: v.cpu().numpy() for k, v in ta.propagate_res_tensors.items()}
    assert np.all(g["outcome"] == int(hyk.taylor_outcome.time_limit))
    assert np.array_equal(np.asarray(ta.state), o.state)
    assert np.array_equal(ta.dtime[0], o.t_hi) and np.array_equal(ta.dtime[1], o.t_lo)
    assert np.array_equal(g["n_steps"], r["n_steps"].astype(np.int64))
    assert np.array_equal(g["min_h"], r["min_h"]) and np.array_equal(g["max_h"], r["max_h"])


@pytest.mark.parametrize("form", ["lane_smem", "team2"])
@pytest.mark.parametrize("name", ["mixed", "consts", "var2"])
def test_ops_step_tc_and_grid_bitwise(oracle, name, form):
    sys_, st, pars, tol, tf = _case(name, n=40)
    ta = hyk.taylor_adaptive_batch(sys_, st, pars=pars, tol=tol, **FORMS[form])
    o = oracle.Oracle(sys_, st, pars=pars, order=ta.order, mode=1)
    for _ in range(2):
        ta.step(write_tc=True)
        _, h = o.step()
        assert np.array_equal(np.asarray(ta.state), o.state)
        assert np.array_equal(np.array([x[1] for x in ta.step_res]), h)
        assert np.array_equal(ta.tc, o.tc)
    grid = np.repeat(ta.time.reshape(1, -1), 12, axis=0) + np.linspace(0.0, 0.5 * tf, 12).reshape(-1, 1)
    _, out = ta.propagate_grid(grid)
    r = o.propagate_grid(grid)
    assert np.array_equal(out, r["grid"])
    assert np.array_equal(np.asarray(ta.state), o.state)
