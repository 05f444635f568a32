"""The compiled CPU stepper (the timed CPU baseline) computes the oracle's
reference ("pin") arithmetic bit for bit.

oracle/cpu_batch.py compiles the code generator's recurrences in the
reference's arithmetic over vector batches of lanes with the oracle's batch
propagate loop; the bench times it as the stand-in for the reference's
compiled batch stepper.  Its states, step counts, min/max step sizes and
outcomes must equal the oracle interpreter's in pin arithmetic for every
batch width (lanes of a batch are padded at the end of the ensemble)."""

import numpy as np
import pytest

import hyk
import systems
from hyk import workloads as W


def _cases():
    rng = np.random.default_rng(5)
    n = 37  # not a multiple of the batch widths
    return {
        "pendulum": (W.pendulum_sys(), W.pendulum_ics(n, seed=1), None, 20, 10.0),
        "kepler": (W.kepler_sys(), W.kepler_ics(n, seed=2), None, 19, 10.0),
        "cr3bp": (W.cr3bp_sys(),) + W.cr3bp_ics(n, seed=3) + (19, 5.0),
        "oss": (W.oss_sys(), W.oss_ics(n, seed=4)[0], None, 19, 2000.0),
        "consts": (systems.consts(), np.vstack([rng.uniform(0.1, 0.3, n), rng.uniform(0.4, 0.6, n)]),
                   np.vstack([rng.uniform(0.1, 0.3, n), rng.uniform(0.3, 0.6, n)]), 15, 1.0),
    }


@pytest.mark.parametrize("batch", [2, 4])
@pytest.mark.parametrize("name", ["pendulum", "kepler", "cr3bp", "oss", "consts"])
def test_cpu_stepper_equals_oracle_pin_arithmetic(oracle, libhyk, name, batch):
    import cpu_batch

    sys_, st, pars, order, tf = _cases()[name]
    r = cpu_batch.ensemble_until(sys_, st, pars, 0.0, tf, order=order, batch=batch, n_threads=2)
    for b in range(0, st.shape[1], 8):
        sl = slice(b, min(b + 8, st.shape[1]))
        o = oracle.Oracle(sys_, st[:, sl], pars=None if pars is None else pars[:, sl], order=order, mode=0)
        ro = o.propagate_until(tf)
        assert np.array_equal(r["state"][:, sl], o.state), name
        assert np.array_equal(r["n_steps"][sl], ro["n_steps"]), name
        assert np.array_equal(r["min_h"][sl], ro["min_h"]) and np.array_equal(r["max_h"][sl], ro["max_h"]), name
        assert np.all(r["outcome"][sl] == int(hyk.taylor_outcome.time_limit))


def test_cpu_peak_probe_runs():
    import cpu_batch

    assert cpu_batch.fp64_peak(1, 0.05) > 1e8
