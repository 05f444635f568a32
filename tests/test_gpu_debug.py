"""The debug build of the kernels (debug=True / HYK_CFG_DEBUG): findings are
recorded, nothing traps, and the results are those of the release build."""

import numpy as np
import pytest
import torch

import hyk
from hyk import workloads as W

pytestmark = pytest.mark.gpu


def test_debug_build_same_results_and_clean_record(libhyk):
    st = W.kepler_ics(256, seed=41)
    a = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15, debug=True)
    b = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    a.propagate_until(10.0)
    b.propagate_until(10.0)
    assert np.array_equal(np.asarray(a.state), np.asarray(b.state))
    assert a.propagate_res == b.propagate_res
    rec = a.debug_record(clear=True)
    assert rec == {"codes": [], "count": 0, "first": None}
    with pytest.raises(ValueError):
        b.debug_record()


def test_debug_records_first_nonfinite_coefficient(libhyk):
    x = hyk.make_vars("x")
    st = np.array([[1.0, 2.0, -1.0, 3.0]])  # sqrt of a negative number in lane 2
    ta = hyk.taylor_adaptive_batch([(x, hyk.sqrt(x))], st, tol=1e-15, debug=True, batch_semantics="lane")
    ta.propagate_until(0.5)
    rec = ta.debug_record(clear=True)
    assert "nonfinite_jet" in rec["codes"] and rec["count"] >= 1
    assert rec["first"] == {"code": "nonfinite_jet", "lane": 2, "variable": 0, "order": 1, "iteration": 0}
    assert ta.propagate_res_tensors["outcome"][2].item() == int(hyk.taylor_outcome.err_nf_state)
    assert ta.debug_record()["count"] == 0  # cleared


def test_debug_records_lane_index_out_of_range(libhyk):
    st = W.kepler_ics(64, seed=42)
    ta = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15, debug=True)
    ref = hyk.taylor_adaptive_batch(W.kepler_sys(), st, tol=1e-15)
    ref.propagate_until(2.0)
    # a lane list with one entry past the batch: the kernel skips it (in the
    # release build too) and the debug build records it
    order = torch.cat([torch.arange(64, device="cuda"), torch.tensor([64 + 5], device="cuda")])
    tf = torch.full((64,), 2.0, dtype=torch.float64, device="cuda")
    ta._run(tf, None, 0, ta._check_prop_args([], None), lane_order=order)
    assert np.array_equal(np.asarray(ta.state), np.asarray(ref.state))
    rec = ta.debug_record(clear=True)
    assert rec["codes"] == ["lane_range"]
    assert rec["first"]["index"] == 69 and rec["first"]["n_lanes"] == 64 and rec["first"]["position"] == 64
