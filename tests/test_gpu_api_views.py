"""Host views of the integrator (heyoka/_test_batch_integrator.py
test_update_d_output, test_dtime, test_set_time, test_type_conversions,
test_llvm_state_settings): read-only, keeping the integrator alive, in both
precisions."""

from copy import deepcopy
from sys import getrefcount

import numpy as np
import pytest

import hyk

pytestmark = pytest.mark.gpu


def _sys():
    x, v = hyk.make_vars("x", "v")
    return [(x, v), (v, -9.8 * hyk.sin(x))]


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_d_output_views(fp_t):
    ta = hyk.taylor_adaptive_batch(_sys(), np.array([[0.0, 0.1, 0.2, 0.3], [0.25, 0.26, 0.27, 0.28]], dtype=fp_t),
                                   fp_type=fp_t)
    ta.step(write_tc=True)
    with pytest.raises(ValueError):
        ta.update_d_output(fp_t(0.3))[0] = fp_t(0.5)
    assert ta.update_d_output(fp_t(0.3)).shape == (2, 4)
    rc = getrefcount(ta)
    tmp = ta.update_d_output(fp_t(0.2))  # noqa: F841
    assert getrefcount(ta) == rc + 1
    with pytest.raises(ValueError):
        ta.update_d_output(np.array([0.3, 0.4, 0.45, 0.46], dtype=fp_t))[0] = fp_t(0.5)
    rc = getrefcount(ta)
    tmp2 = ta.update_d_output(np.array([0.31, 0.41, 0.66, 0.67], dtype=fp_t))  # noqa: F841
    assert getrefcount(ta) == rc + 1
    cp = deepcopy(ta.update_d_output(fp_t(0.3)))
    assert np.all(cp == ta.update_d_output([fp_t(0.3)] * 4))
    ta.set_time(fp_t(0.0))
    ta.state[:] = [[0.0, 0.01, 0.02, 0.03], [0.205, 0.206, 0.207, 0.208]]
    ta.step(write_tc=True)
    eps = np.finfo(fp_t).eps * 10
    ta.update_d_output(ta.time)
    assert np.allclose(ta.d_output, np.asarray(ta.state), rtol=eps, atol=eps)
    ta.update_d_output(fp_t(0.0), rel_time=True)
    assert np.allclose(ta.d_output, np.asarray(ta.state), rtol=eps, atol=eps)


@pytest.mark.parametrize("fp_t", [np.float32, float])
def test_time_views_and_dtime(fp_t):
    ta = hyk.taylor_adaptive_batch(_sys(), np.array([[0.0, 0.1], [0.25, 0.26]], dtype=fp_t), fp_type=fp_t)
    assert np.all(ta.time == [0, 0])
    rc = getrefcount(ta)
    t = ta.time  # noqa: F841
    assert getrefcount(ta) == rc + 1
    ta.set_time([fp_t(-1.0), fp_t(1.0)])
    assert np.all(ta.time == [-1, 1])
    ta.set_time(fp_t(5.0))
    assert np.all(ta.time == [5, 5])
    ta.set_time(fp_t(0.0))
    with pytest.raises(ValueError):
        ta.dtime[0][0] = 0.5
    with pytest.raises(ValueError):
        ta.dtime[1][0] = 0.5
    ta.step()
    ta.propagate_for(fp_t(1000.1))
    assert not np.all(ta.dtime[1] == [0, 0])
    ta.set_dtime(fp_t(1.0), fp_t(0.5))
    assert np.all(ta.dtime[0] == [1.5, 1.5]) and np.all(ta.dtime[1] == [0, 0])
    ta.set_dtime([fp_t(1.0), fp_t(2.0)], [fp_t(0.5), fp_t(0.25)])
    assert np.all(ta.dtime[0] == [1.5, 2.25]) and np.all(ta.dtime[1] == [0, 0])
    with pytest.raises(TypeError, match="must be of the same type"):
        ta.set_dtime([fp_t(1.0), fp_t(2.0)], fp_t(0.5))


def test_type_conversions_and_llvm_state():
    ta = hyk.taylor_adaptive_batch(_sys(), ((0.0, 0.1), (0.25, 0.26)), tol=1e-4)
    assert np.all(ta.state == ((0.0, 0.1), (0.25, 0.26)))
    if np.finfo(np.longdouble).nmant != np.finfo(np.double).nmant:
        ld = np.longdouble
        with pytest.raises(TypeError):
            hyk.taylor_adaptive_batch(_sys(), ((ld(0.0), ld(0.1)), (ld(0.25), ld(0.26))), tol=1e-4)
        with pytest.raises(TypeError):
            hyk.taylor_adaptive_batch(_sys(), np.array([[0.0, 0.1], [0.25, 0.26]], dtype=ld), tol=1e-4)
    rc = getrefcount(ta)
    tmp = ta.llvm_state  # noqa: F841
    assert getrefcount(ta) == rc + 1
    assert not ta.llvm_state.force_avx512 and not ta.llvm_state.slp_vectorize
    with pytest.warns(UserWarning):
        ta = hyk.taylor_adaptive_batch(_sys(), [[0.0, 0.0], [0.0, 0.0]], force_avx512=True, slp_vectorize=True,
                                       parjit=True, compact_mode=True, code_model=hyk.code_model.large)
    assert ta.llvm_state.force_avx512 and ta.llvm_state.slp_vectorize
    assert ta.llvm_state.code_model == hyk.code_model.large
