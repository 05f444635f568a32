"""Model factories used by the batch-integrator workloads.

Restatements of the reference's expression factories (exposed at
heyoka/expose_models.cpp:237-242 nbody, :275-278 pendulum, :395-397 cr3bp,
re-exported by heyoka/model/__init__.py:13-25).  The state layouts are the
ones pinned by the reference's tests (heyoka/_test_model.py:153-278):

* ``pendulum``: ``[x, v]``, ``x' = v``, ``v' = -(gconst/length) * sin(x)``.
* ``nbody``: per body ``[x_i, y_i, z_i, vx_i, vy_i, vz_i]``; velocities'
  derivatives are sums over the other bodies of ``G m_j (r_j - r_i) / |r_j - r_i|^3``.
  Each pair (i < j) builds its separation, ``|r|^-3`` once, and feeds both
  bodies; massless bodies do not attract.
* ``cr3bp``: rotating-frame Hamiltonian form, state ``[x, y, z, px, py, pz]``
  with the primaries (1 - mu) at x = mu and mu at x = mu - 1, as written in
  doc/notebooks/Periodic orbits in the CR3BP.ipynb.  ``mu`` may be a number
  or an expression such as ``par[0]``.
* ``kepler`` (not a reference model; the two-body workload of this package):
  ``r'' = -mu r / |r|^3`` written as ``-x * (x**2 + y**2 + z**2)**-1.5``.
"""

from __future__ import annotations

from . import expr as _e


def pendulum(gconst=1.0, length=1.0):
    x, v = _e.make_vars("x", "v")
    k = _e._ex(gconst) / _e._ex(length)
    if k.is_number and k.value == 1.0:
        return [(x, v), (v, -_e.sin(x))]
    return [(x, v), (v, (-k) * _e.sin(x))]


def pendulum_energy(gconst=1.0, length=1.0):
    x, v = _e.make_vars("x", "v")
    g, l = _e._ex(gconst), _e._ex(length)
    return (0.5 * l * l) * v**2 + (g * l) * (1.0 - _e.cos(x))


def nbody(n, Gconst=1.0, masses=None):
    if n < 2:
        raise ValueError("Cannot construct an N-body system with N == {}".format(n))
    masses = [1.0] * n if masses is None else list(masses)
    if len(masses) > n:
        raise ValueError(
            "In an N-body system the number of particles with mass ({}) cannot be "
            "greater than the number of particles ({})".format(len(masses), n)
        )
    masses = [_e._ex(m) for m in masses] + [_e.expression(0.0)] * (n - len(masses))
    G = _e._ex(Gconst)
    xs, ys, zs, vxs, vys, vzs = [], [], [], [], [], []
    for i in range(n):
        x, y, z, vx, vy, vz = _e.make_vars(
            "x_{}".format(i), "y_{}".format(i), "z_{}".format(i),
            "vx_{}".format(i), "vy_{}".format(i), "vz_{}".format(i),
        )
        xs.append(x), ys.append(y), zs.append(z), vxs.append(vx), vys.append(vy), vzs.append(vz)
    acc = [[[], [], []] for _ in range(n)]
    Gm = [G * m for m in masses]
    for i in range(n):
        for j in range(i + 1, n):
            mi_zero = masses[i].is_number and masses[i].value == 0.0
            mj_zero = masses[j].is_number and masses[j].value == 0.0
            if mi_zero and mj_zero:
                continue
            dx, dy, dz = xs[j] - xs[i], ys[j] - ys[i], zs[j] - zs[i]
            r_m3 = (_e.square(dx) + _e.square(dy) + _e.square(dz)) ** -1.5
            for k, d in enumerate((dx, dy, dz)):
                t = d * r_m3
                if not mj_zero:
                    acc[i][k].append(Gm[j] * t)
                if not mi_zero:
                    acc[j][k].append(-(Gm[i] * t))
    sys = []
    for i in range(n):
        sys += [(xs[i], vxs[i]), (ys[i], vys[i]), (zs[i], vzs[i])]
        for k, v in enumerate((vxs[i], vys[i], vzs[i])):
            sys.append((v, _e.sum(acc[i][k])))
    return sys


def cr3bp(mu=1e-3):
    x, y, z, px, py, pz = _e.make_vars("x", "y", "z", "px", "py", "pz")
    mu = _e._ex(mu)
    rps_32 = ((x - mu) ** 2 + y**2 + z**2) ** -1.5
    rpj_32 = ((x - mu + 1.0) ** 2 + y**2 + z**2) ** -1.5
    return [
        (x, px + y),
        (y, py - x),
        (z, pz),
        (px, py - (1.0 - mu) * rps_32 * (x - mu) - mu * rpj_32 * (x - mu + 1.0)),
        (py, -px - ((1.0 - mu) * rps_32 + mu * rpj_32) * y),
        (pz, -((1.0 - mu) * rps_32 + mu * rpj_32) * z),
    ]


def cr3bp_jacobi(mu=1e-3):
    x, y, z, px, py, pz = _e.make_vars("x", "y", "z", "px", "py", "pz")
    mu = _e._ex(mu)
    vx, vy, vz = px + y, py - x, pz
    r1 = _e.sqrt((x - mu) ** 2 + y**2 + z**2)
    r2 = _e.sqrt((x - mu + 1.0) ** 2 + y**2 + z**2)
    omega = 0.5 * (x**2 + y**2) + (1.0 - mu) / r1 + mu / r2
    return omega - 0.5 * (vx**2 + vy**2 + vz**2)


def kepler(mu=1.0):
    x, y, z, vx, vy, vz = _e.make_vars("x", "y", "z", "vx", "vy", "vz")
    mu = _e._ex(mu)
    r_m3 = (x**2 + y**2 + z**2) ** -1.5
    return [
        (x, vx),
        (y, vy),
        (z, vz),
        (vx, -mu * x * r_m3 if not (mu.is_number and mu.value == 1.0) else -x * r_m3),
        (vy, -mu * y * r_m3 if not (mu.is_number and mu.value == 1.0) else -y * r_m3),
        (vz, -mu * z * r_m3 if not (mu.is_number and mu.value == 1.0) else -z * r_m3),
    ]
