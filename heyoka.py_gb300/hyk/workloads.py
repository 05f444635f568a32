"""Seeded synthetic ensembles with the shapes and distributions of the
integrator's benchmark workloads (initial conditions only; no data files).

* pendulum: x0 ~ U[-1.5, 1.5] rad, v0 ~ U[-0.5, 0.5], x' = v, v' = -9.8 sin x.
* kepler: mu = 1, a ~ U[0.5, 2], e ~ U[0, 0.6], i ~ U[0, pi/4],
  Omega, omega, M ~ U[0, 2 pi), converted to Cartesian state.
* cr3bp: mu ~ U[0.005, 0.02] per lane (par[0]), states near L4 =
  (mu - 1/2, sqrt(3)/2, 0) with momenta p = v + (-y, x, 0), position noise
  sigma 1e-3 and velocity noise sigma 1e-4.
* outer solar system: Sun plus 5 bodies on circular coplanar orbits, each
  state component scaled by (1 + 1e-6 N(0, 1)).
"""

from __future__ import annotations

import math

import numpy as np

from . import expr as _e
from . import model as _m


def pendulum_sys():
    x, v = _e.make_vars("x", "v")
    return [(x, v), (v, -9.8 * _e.sin(x))]


def pendulum_ics(n, seed=0):
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(-1.5, 1.5, n)
    v0 = rng.uniform(-0.5, 0.5, n)
    return np.stack([x0, v0])


def kepler_sys():
    return _m.kepler(1.0)


def kepler_elements_to_cartesian(a, e, inc, Om, om, M, mu=1.0):
    E = M.copy()
    for _ in range(60):
        f = E - e * np.sin(E) - M
        dE = f / (1.0 - e * np.cos(E))
        E = E - dE
        if np.max(np.abs(dE)) < 1e-15:
            break
    cE, sE = np.cos(E), np.sin(E)
    b = a * np.sqrt(1.0 - e * e)
    xp, yp = a * (cE - e), b * sE
    n = np.sqrt(mu / a**3)
    rr = 1.0 - e * cE
    vxp, vyp = -a * n * sE / rr, b * n * cE / rr
    cO, sO, co, so, ci, si = np.cos(Om), np.sin(Om), np.cos(om), np.sin(om), np.cos(inc), np.sin(inc)
    r11, r12 = cO * co - sO * so * ci, -cO * so - sO * co * ci
    r21, r22 = sO * co + cO * so * ci, -sO * so + cO * co * ci
    r31, r32 = so * si, co * si
    x, y, z = r11 * xp + r12 * yp, r21 * xp + r22 * yp, r31 * xp + r32 * yp
    vx, vy, vz = r11 * vxp + r12 * vyp, r21 * vxp + r22 * vyp, r31 * vxp + r32 * vyp
    return np.stack([x, y, z, vx, vy, vz])


def kepler_ics(n, seed=1):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.5, 2.0, n)
    e = rng.uniform(0.0, 0.6, n)
    inc = rng.uniform(0.0, math.pi / 4, n)
    Om = rng.uniform(0.0, 2 * math.pi, n)
    om = rng.uniform(0.0, 2 * math.pi, n)
    M = rng.uniform(0.0, 2 * math.pi, n)
    return kepler_elements_to_cartesian(a, e, inc, Om, om, M)


def cr3bp_sys():
    return _m.cr3bp(_e.par[0])


def cr3bp_ics(n, seed=3):
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.005, 0.02, n)
    x = mu - 0.5 + rng.normal(0.0, 1e-3, n)
    y = math.sqrt(3.0) / 2.0 + rng.normal(0.0, 1e-3, n)
    z = rng.normal(0.0, 1e-3, n)
    vx = rng.normal(0.0, 1e-4, n)
    vy = rng.normal(0.0, 1e-4, n)
    vz = rng.normal(0.0, 1e-4, n)
    st = np.stack([x, y, z, vx - y, vy + x, vz])
    return st, mu.reshape(1, n)


OSS_G = 0.01720209895**2
OSS_MASSES = [1.0, 9.5e-4, 2.9e-4, 4.4e-5, 5.2e-5, 6.6e-9]
OSS_A = [5.2, 9.5, 19.2, 30.1, 39.5]


def oss_sys():
    return _m.nbody(6, Gconst=OSS_G, masses=OSS_MASSES)


def oss_ics(n, seed=2):
    rng = np.random.default_rng(seed)
    base = np.zeros(36)
    for k, a in enumerate(OSS_A):
        ph = 2 * math.pi * k / 5
        v = math.sqrt(OSS_G * (1.0 + OSS_MASSES[k + 1]) / a)
        o = 6 * (k + 1)
        base[o: o + 6] = [a * math.cos(ph), a * math.sin(ph), 0.0, -v * math.sin(ph), v * math.cos(ph), 0.0]
    st = base.reshape(36, 1) * (1.0 + 1e-6 * rng.normal(size=(36, n)))
    t_end = np.exp(rng.uniform(math.log(1e3), math.log(1e5), n))
    return st, t_end


def oss_energy(st):
    """Total energy of outer-solar-system states, shape (36, n)."""
    st = np.asarray(st, dtype=np.float64)
    m = np.asarray(OSS_MASSES).reshape(-1, 1)
    b = st.reshape(6, 6, -1)
    kin = 0.5 * np.sum(m * np.sum(b[:, 3:6] ** 2, axis=1), axis=0)
    pot = np.zeros(st.shape[1])
    for i in range(6):
        for j in range(i + 1, 6):
            r = np.sqrt(np.sum((b[i, 0:3] - b[j, 0:3]) ** 2, axis=0))
            pot -= OSS_G * m[i, 0] * m[j, 0] / r
    return kin + pot
