"""Binary128 reference states of 1024 orbits of the Kepler benchmark ensemble.

The benchmark ensemble is the 2^20 Kepler orbits of ``hyk.workloads.kepler_ics``
(seed 1).  A seeded subsample of 1024 of them (``numpy.random.default_rng(123)``,
without replacement, sorted) is integrated from t = 0 to t = 50 and on to
t = 200 by the oracle in binary128 (``prec=1``) at tol 1e-24 (Taylor order 29),
far below the double-precision runs' errors (a tol 1e-28 run gives the same
doubles).  The states, rounded to double, are written to
``kepler_t200_quad_1024.npz`` next to this script, with the subsample's
indices.  It stands in for the reference's real128 scalar integrator
(heyoka/taylor_expose_integrator.cpp:502-533), which cannot be run here.

Usage: python tests/golden/make_kepler_quad.py [workers]   (about 1 CPU-minute per 100 orbits)
"""

import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (os.path.join(ROOT, "heyoka.py_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N_SAMPLE = 1024
TIMES = (50.0, 200.0)
QUAD_TOL = 1e-24


def subsample_indices(n_total=1 << 20, n=N_SAMPLE):
    return np.sort(np.random.default_rng(123).choice(n_total, n, replace=False))


def _run(st):
    import pyoracle
    from hyk import workloads as W
    from hyk.decompose import order_from_tol

    q = pyoracle.Oracle(W.kepler_sys(), st, order=order_from_tol(QUAD_TOL), prec=1, mode=0)
    out = []
    for t in TIMES:
        q.propagate_until(t)
        out.append(q.state.copy())
    return out


def main(workers):
    from hyk import workloads as W

    idx = subsample_indices()
    st = np.ascontiguousarray(W.kepler_ics(1 << 20, seed=1)[:, idx])
    chunks = [st[:, i:i + 32] for i in range(0, N_SAMPLE, 32)]
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_run, chunks)
    out = {"idx": idx, "times": np.array(TIMES)}
    for k, t in enumerate(TIMES):
        out["state_t{:g}".format(t)] = np.concatenate([r[k] for r in res], axis=1)
    path = os.path.join(HERE, "kepler_t200_quad_1024.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count())
