"""Events on the GPU: the reference's batch event tests (heyoka/test.py:693-1000)
through the hyk API, and bit-for-bit parity of event times, directions,
outcomes and final states with the oracle (same root finder, same
arithmetic)."""

from copy import deepcopy
from sys import getrefcount

import numpy as np
import pytest

import hyk
from hyk import event_direction, nt_event_batch, t_event_batch, taylor_outcome

pytestmark = pytest.mark.gpu


def pend():
    x, v = hyk.make_vars("x", "v")
    return x, v, [(x, v), (v, -9.8 * hyk.sin(x))]


def test_reference_nt_events():
    x, v, sys_ = pend()
    counter = [0] * 2
    cur_time = [0.0] * 2
    ta_id = None

    def cb0(ta, t, d_sgn, bidx):
        assert t > cur_time[bidx]
        assert counter[bidx] % 3 == 0 or counter[bidx] % 3 == 2
        assert ta_id == id(ta)
        counter[bidx] += 1
        cur_time[bidx] = t

    def cb1(ta, t, d_sgn, bidx):
        assert t > cur_time[bidx]
        assert counter[bidx] % 3 == 1
        assert ta_id == id(ta)
        counter[bidx] += 1
        cur_time[bidx] = t

    ta = hyk.taylor_adaptive_batch(sys_, [[0.0, 0.001], [0.25, 0.2501]],
                                   nt_events=[nt_event_batch(v * v - 1e-10, cb0), nt_event_batch(v, cb1)])
    ta_id = id(ta)
    ta.propagate_until([4.0, 4.0])
    assert all(r[0] == taylor_outcome.time_limit for r in ta.propagate_res)
    assert counter == [12, 12]


def test_reference_event_properties_and_copies():
    x, v, sys_ = pend()

    class cbk:
        def __init__(self):
            self.lst = []

        def __call__(self, ta, t, d_sgn, bidx):
            pass

    ta = hyk.taylor_adaptive_batch(sys_, [[0.0, 0.001], [0.25, 0.2501]],
                                   nt_events=[nt_event_batch(v * v - 1e-10, cbk()), nt_event_batch(v, cbk()),
                                              nt_event_batch(v, cbk())])
    rc = getrefcount(ta)
    nt_list = ta.nt_events  # noqa: F841
    assert getrefcount(ta) == rc + 3
    for k in range(3):
        assert id(ta.nt_events[k].callback) == id(ta.nt_events[k].callback)
        assert id(ta.nt_events[k].callback.lst) == id(ta.nt_events[k].callback.lst)
    ta_copy = deepcopy(ta)
    for k in range(3):
        assert id(ta_copy.nt_events[k].callback) != id(ta.nt_events[k].callback)
        assert id(ta_copy.nt_events[k].callback.lst) != id(ta.nt_events[k].callback.lst)


def test_reference_callback_errors():
    x, v, sys_ = pend()

    def cb2(ta, t):
        pass

    ta = hyk.taylor_adaptive_batch(sys_, [[0.0, 0.001], [0.25, 0.2501]], nt_events=[nt_event_batch(v * v - 1e-10, cb2)])
    with pytest.raises(RuntimeError):
        ta.propagate_until([4.0, 4.0])
    ta = hyk.taylor_adaptive_batch(sys_, [[0.0, 0.001], [0.25, 0.2501]],
                                   t_events=[t_event_batch(v * v - 1e-10, callback=cb2)])
    with pytest.raises(RuntimeError):
        ta.propagate_until([4.0, 4.0])

    def cb3(ta, d_sgn, bidx):
        return "hello"

    ta = hyk.taylor_adaptive_batch(sys_, [[0.0, 0.001], [0.25, 0.2501]],
                                   t_events=[t_event_batch(v * v - 1e-10, callback=cb3)])
    with pytest.raises(RuntimeError) as ei:
        ta.propagate_until([4.0, 4.0])
    assert "in the construction of the return value of an event callback" in str(ei.value)


def test_reference_terminal_events_with_step():
    x, v, sys_ = pend()
    counter_t = [0] * 2
    counter_nt = [0] * 2
    cur_time = [0.0] * 2
    ta_id = None

    def cb0(ta, t, d_sgn, bidx):
        assert t > cur_time[bidx]
        assert ta_id == id(ta)
        counter_nt[bidx] += 1
        cur_time[bidx] = t

    def cb1(ta, d_sgn, bidx):
        assert ta.time[bidx] > cur_time[bidx]
        assert ta_id == id(ta)
        counter_t[bidx] += 1
        cur_time[bidx] = ta.time[bidx]
        return True

    ta = hyk.taylor_adaptive_batch(sys_, [[0.0, 0.001], [0.25, 0.2501]],
                                   nt_events=[nt_event_batch(v * v - 1e-10, cb0)],
                                   t_events=[t_event_batch(v, callback=cb1)])
    ta_id = id(ta)
    while True:
        ta.step()
        if all(r[0] > taylor_outcome.success for r in ta.step_res):
            break
    assert all(int(r[0]) == 0 for r in ta.step_res)
    assert all(t < 1 for t in ta.time)
    assert counter_nt == [1, 1] and counter_t == [1, 1]
    while True:
        ta.step()
        if all(r[0] > taylor_outcome.success for r in ta.step_res):
            break
    assert all(int(r[0]) == 0 for r in ta.step_res)
    assert all(t > 1 for t in ta.time)
    assert counter_nt == [3, 3] and counter_t == [2, 2]


def _ics(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-1.2, 1.2, n), rng.uniform(-0.5, 0.5, n)])


@pytest.mark.parametrize("mode", ["persistent", "plain"])
def test_nt_events_bitwise_vs_oracle(oracle, mode):
    x, v, sys_ = pend()
    st = _ics(96, 41)
    recs = []

    def cb_a(ta, t, d_sgn, bidx):
        recs.append((bidx, 0, t, d_sgn))

    def cb_b(ta, t, d_sgn, bidx):
        recs.append((bidx, 1, t, d_sgn))

    ta = hyk.taylor_adaptive_batch(sys_, st, prop_mode=mode,
                                   nt_events=[nt_event_batch(v * v - 1e-4, cb_a),
                                              nt_event_batch(x, cb_b, direction=event_direction.positive)])
    ta.propagate_until(7.5)
    r = oracle.propagate_ev(sys_, [(v * v - 1e-4, False, 0, -1.0), (x, False, 1, -1.0)], st, 7.5, order=ta.order)
    assert np.array_equal(np.asarray(ta.state), r["state"])
    assert np.array_equal(ta.time, r["t_hi"])
    assert np.array_equal(ta.propagate_res_tensors["n_steps"].cpu().numpy(), r["n_steps"].astype(np.int64))
    got = sorted(recs)
    want = sorted((int(l), int(i) >> 2, float(t), (int(i) & 3) - 1)
                  for l, i, t in zip(r["rec_lane"], r["rec_info"], r["rec_t_hi"]))
    assert len(got) == len(want) > 96
    assert got == want


def test_terminal_events_bitwise_vs_oracle(oracle):
    x, v, sys_ = pend()
    st = _ics(80, 42)
    ta = hyk.taylor_adaptive_batch(sys_, st, t_events=[t_event_batch(v, direction=event_direction.negative)])
    ta.propagate_until(20.0)
    r = oracle.propagate_ev(sys_, [(v, True, -1, -1.0)], st, 20.0, order=ta.order)
    assert [int(o) for o, *_ in ta.propagate_res] == list(r["outcome"])
    assert np.array_equal(np.asarray(ta.state), r["state"])
    assert np.array_equal(ta.time, r["t_hi"])
    # continue: the cooldown keeps the lanes from stopping at the same root
    ta.propagate_until(20.0)
    r2 = oracle.propagate_ev(sys_, [(v, True, -1, -1.0)], r["state"], 20.0, order=ta.order, time=r["t_hi"],
                             time_lo=r["t_lo"], ev_last=r["ev_last"])
    assert np.array_equal(ta.time, r2["t_hi"])
    assert np.array_equal(np.asarray(ta.state), r2["state"])
    assert np.all(ta.time > r["t_hi"])


def test_reference_propagate_outcome_and_cooldowns():
    """heyoka/_test_batch_integrator.py:560-600: a terminal event without
    callback stops propagate_until with outcome -1; te_cooldowns and
    reset_cooldowns per lane."""
    x, v, sys_ = pend()

    def cb0(ta, t, d_sgn, bidx):
        pass

    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0.0, 0.001], [0.25, 0.2501]]),
                                   nt_events=[nt_event_batch(v * v - 1e-6, cb0)], t_events=[t_event_batch(v)])
    assert ta.with_events and len(ta.t_events) == 1 and len(ta.nt_events) == 1
    ta.propagate_until([1e9, 1e9])
    assert all(int(r[0]) == -1 for r in ta.propagate_res)
    assert ta.te_cooldowns[0][0] is not None and ta.te_cooldowns[1][0] is not None
    ta.reset_cooldowns(0)
    assert ta.te_cooldowns[0][0] is None and ta.te_cooldowns[1][0] is not None
    ta.reset_cooldowns()
    assert ta.te_cooldowns[0][0] is None and ta.te_cooldowns[1][0] is None


def _nt_noop(ta, t, d_sgn, bidx):
    pass


class _Counting:
    """A stateful terminal callback (module level, so that plain pickle
    serialises it where cloudpickle is not installed)."""

    def __init__(self):
        self.n = 0

    def __call__(self, ta, d_sgn, bidx):
        self.n += 1
        return True


def test_reference_event_pickling():
    """heyoka/_test_batch_integrator.py:605-690: integrators with events
    survive pickling, stateful callbacks included."""
    import pickle

    x, v, sys_ = pend()
    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0, 0.01], [0.25, 0.26]]),
                                   nt_events=[nt_event_batch(v * v - 1e-6, _nt_noop)])
    for _ in range(4):
        ta.step()
    ta2 = pickle.loads(pickle.dumps(ta))
    assert np.all(np.asarray(ta.state) == np.asarray(ta2.state)) and np.all(ta.time == ta2.time)
    assert len(ta.nt_events) == len(ta2.nt_events)
    ta.step()
    ta2.step()
    assert np.all(np.asarray(ta.state) == np.asarray(ta2.state))

    clb = _Counting()
    ta = hyk.taylor_adaptive_batch(sys_, np.array([[0, 0.01], [0.25, 0.26]]),
                                   t_events=[t_event_batch(v, callback=clb)])
    assert id(clb) != id(ta.t_events[0].callback) and ta.t_events[0].callback.n == 0
    ta.propagate_until([100.0, 100.0])
    assert ta.t_events[0].callback.n > 0
    ta2 = pickle.loads(pickle.dumps(ta))
    assert ta.t_events[0].callback.n == ta2.t_events[0].callback.n


def test_events_with_global_memory_coefficients(oracle):
    """Events in the lane form with its coefficients in global memory (the
    form CR3BP-sized systems get): the same roots and states as the oracle."""
    x, v, sys_ = pend()
    st = _ics(64, 43)
    recs = []

    def cb(ta, t, d_sgn, bidx):
        recs.append((bidx, t, d_sgn))

    ta = hyk.taylor_adaptive_batch(sys_, st, global_jets=True, nt_events=[nt_event_batch(v, cb)],
                                   t_events=[t_event_batch(x - 0.5, direction=event_direction.positive)])
    assert ta.module_info["smem_per_lane"] == 0
    ta.propagate_until(6.0)
    r = oracle.propagate_ev(sys_, [(x - 0.5, True, 1, -1.0), (v, False, 0, -1.0)], st, 6.0, order=ta.order)
    assert np.array_equal(np.asarray(ta.state), r["state"])
    assert np.array_equal(ta.time, r["t_hi"])
    assert [int(o) for o, *_ in ta.propagate_res] == list(r["outcome"])
    want = sorted((int(l), float(t), (int(i) & 3) - 1) for l, i, t in zip(r["rec_lane"], r["rec_info"], r["rec_t_hi"]))
    assert sorted(recs) == want
