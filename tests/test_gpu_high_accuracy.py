"""High-accuracy mode (the reference's ``high_accuracy=True``: the state
update by compensated summation instead of Horner's rule) on the GPU, bit for
bit against the oracle's high-accuracy gpu arithmetic, in both kernel forms."""

import numpy as np
import pytest

import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("team", [1, 4])
def test_high_accuracy_bitwise(oracle, team):
    st = W.kepler_ics(64, seed=51)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15, high_accuracy=True, team_size=team)
    assert ta.high_accuracy
    ta.propagate_until(30.0)
    o = oracle.Oracle(W.kepler_sys(), st, order=ta.order, mode=3)
    o.propagate_until(30.0)
    assert np.array_equal(np.asarray(ta.state), o.state)
    plain = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15, team_size=team)
    plain.propagate_until(30.0)
    assert not np.array_equal(np.asarray(plain.state), np.asarray(ta.state))
    assert np.max(np.abs(np.asarray(plain.state) - np.asarray(ta.state))) < 1e-11


@pytest.mark.parametrize("team", [1, 4])
def test_high_accuracy_float32_bitwise(oracle, team):
    """The reference's basic test constructs float32 integrators with
    high_accuracy=True; the compensated update in single precision matches
    the oracle's float arithmetic bit for bit."""
    st = W.kepler_ics(64, seed=52).astype(np.float32)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, high_accuracy=True, team_size=team, fp_type=np.float32)
    assert ta.high_accuracy and ta.order == 9
    ta.propagate_until(10.0)
    o = oracle.Oracle(W.kepler_sys(), st.astype(np.float64), order=ta.order, prec=2, mode=3)
    o.propagate_until(10.0)
    assert np.array_equal(np.asarray(ta.state).astype(np.float64), o.state)
