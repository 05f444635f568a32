"""The reference's whole-batch rules on the GPU (batch_semantics).

In the reference's batch propagate loop a state that becomes non-finite
stops every lane of the batch at that iteration: the lane concerned reports
err_nf_state and the others the outcome of their last step, with their
state, time and step count as of that iteration
(heyoka/expose_batch_integrators.cpp:279-314; restated in the oracle's batch
loop).  That is the default here (batch_semantics="reference"), in every
propagation form: the one-launch-per-step form steps the lanes in lockstep;
the persistent form, whose lanes run ahead of one another, propagates again
from the initial state when a lane failed.  batch_semantics="lane" keeps a
failure to its own lane.  Event callbacks run after each batch step under
the reference semantics, so a callback sees the integrator at the end of the
step in which its event fell."""

import numpy as np
import pytest
import torch

import hyk

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(libhyk):
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    yield


def blowup():
    """x' = x^2 overflows at t = 1/x0 (lane 0: at its 242nd iteration); v is
    driven by cos(10 t), so the other lanes take ~0.12 time units per step."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, x * x), (v, hyk.cos(10.0 * hyk.time) - v)]
    st = np.array([[1.0, 0.001, 0.0012, 0.0011, 0.00105, 0.0013], [0.0, 0.1, 0.2, 0.3, 0.4, 0.5]])
    tf = np.array([3.0, 100.0, 80.0, 1.0, 94.0, 60.0])
    return sys_, st, tf


def immediate():
    """log of a negative number: lane 0 is non-finite after its first step."""
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, hyk.log(x))], np.array([[-1.0, 1.0, 2.0, 1.5], [0.0, 0.0, 0.1, 0.2]]), np.full(4, 0.5)


FORMS = {"persistent": dict(prop_mode="persistent"), "plain": dict(prop_mode="plain"),
         "team2": dict(team_size=2), "team2_plain": dict(team_size=2, prop_mode="plain")}


def _res(ta):
    r = ta.propagate_res_tensors
    return {k: v.cpu().numpy() for k, v in r.items()}


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("case", ["blowup", "immediate"])
def test_non_finite_state_stops_the_batch(oracle, case, form):
    sys_, st, tf = {"blowup": blowup, "immediate": immediate}[case]()
    ta = hyk.taylor_adaptive_batch(sys_, st, **FORMS[form])
    ta.propagate_until(tf)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    r = o.propagate_until(tf)
    g = _res(ta)
    assert np.array_equal(g["outcome"], r["outcome"].astype(np.int64))
    assert g["outcome"][0] == int(hyk.taylor_outcome.err_nf_state)
    assert np.array_equal(np.asarray(ta.state), o.state, equal_nan=True)
    assert np.array_equal(ta.dtime[0], o.t_hi, equal_nan=True)
    assert np.array_equal(g["n_steps"], r["n_steps"].astype(np.int64))
    ok = ~np.isnan(r["min_h"])
    assert np.array_equal(g["min_h"][ok], r["min_h"][ok]) and np.array_equal(g["max_h"][ok], r["max_h"][ok])
    if case == "blowup":
        # the long lanes stopped at the failing iteration, far from their end time
        assert np.all(ta.time[[1, 2, 4, 5]] < 40.0)
        assert np.all(g["outcome"][[1, 2, 4, 5]] == int(hyk.taylor_outcome.success))


@pytest.mark.parametrize("form", ["persistent", "plain"])
def test_lane_semantics_opt_in(form):
    sys_, st, tf = blowup()
    ta = hyk.taylor_adaptive_batch(sys_, st, batch_semantics="lane", **FORMS[form])
    ta.propagate_until(tf)
    g = _res(ta)
    assert g["outcome"][0] == int(hyk.taylor_outcome.err_nf_state)
    assert np.all(g["outcome"][1:] == int(hyk.taylor_outcome.time_limit))
    assert np.array_equal(ta.time[1:], tf[1:])
    with pytest.raises(ValueError, match="batch_semantics"):
        hyk.taylor_adaptive_batch(sys_, st, batch_semantics="nope")


def test_grid_and_c_output_after_batch_stop(oracle):
    sys_, st, tf = blowup()
    grid = np.linspace(0.0, 1.0, 9).reshape(-1, 1) * tf.reshape(1, -1)
    ta = hyk.taylor_adaptive_batch(sys_, st)
    _, out = ta.propagate_grid(grid)
    o = oracle.Oracle(sys_, st, order=ta.order, mode=1)
    r = o.propagate_grid(grid)
    assert np.array_equal(out, r["grid"], equal_nan=True)
    # rows after the stop are NaN (the reference fills unreached rows with NaN)
    assert np.isnan(out[-1, :, 1]).all()
    tb = hyk.taylor_adaptive_batch(sys_, st)
    c, _ = tb.propagate_until(tf, c_output=True)
    o = oracle.Oracle(sys_, st, order=tb.order, mode=1)
    rc = o.propagate_until(tf, c_output=True)
    # the failing iteration is recorded for no lane
    assert c.n_steps == rc["c_tcs"].shape[0]
    assert np.array_equal(c.tcs, rc["c_tcs"])


def test_ensemble_iteration_stops_alone(oracle):
    """In an ensemble each iteration is its own batch: a failure stops the
    lanes of its iteration only."""
    sys_, st, tf = blowup()
    st4 = st[:, [0, 1, 2, 4]]
    ta = hyk.taylor_adaptive_batch(sys_, st4)

    def gen(t, i):
        t.state[:] = st4 if i == 1 else st4[:, [1, 1, 2, 3]]
        return t

    ret = hyk.ensemble_propagate_until(ta, 50.0, 3, gen)
    res = [[r[0] for r in x[0].propagate_res] for x in ret]
    assert res[1][0] == hyk.taylor_outcome.err_nf_state
    assert all(oc == hyk.taylor_outcome.success for oc in res[1][1:])
    assert all(oc == hyk.taylor_outcome.time_limit for i in (0, 2) for oc in res[i])
    o = oracle.Oracle(sys_, st4, order=ta.order, mode=1)
    o.propagate_until(50.0)
    assert np.array_equal(np.asarray(ret[1][0].state), o.state, equal_nan=True)


def test_nt_event_callbacks_see_the_end_of_their_step():
    """Non-terminal event callbacks run after each batch step: the integrator
    a callback receives is at the end of the step that contains the event."""
    x, v = hyk.make_vars("x", "v")
    sys_ = [(x, v), (v, -9.8 * hyk.sin(x))]
    seen = []

    def cb(ta, t, d, b):
        seen.append((b, t, float(ta.time[b])))

    st = np.array([[0.3, 0.5], [0.0, 0.0]])
    ta = hyk.taylor_adaptive_batch(sys_, st, nt_events=[hyk.nt_event_batch(v, cb)])
    ta.propagate_until(10.0)
    assert len(seen) > 8
    for b, t, now in seen:
        assert now >= t and now < t + 0.5  # within one step of the event
    assert len({now for _, _, now in seen}) > 4  # not all at the final time
    tl = hyk.taylor_adaptive_batch(sys_, st, nt_events=[hyk.nt_event_batch(v, cb)], batch_semantics="lane")
    seen.clear()
    tl.propagate_until(10.0)
    assert all(now == 10.0 for _, _, now in seen)
