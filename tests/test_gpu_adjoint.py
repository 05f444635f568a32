"""Discrete adjoint (taylor_flow) against central finite differences and
against first-order variational equations (the reference's var_ode_sys
sensitivities, restated)."""

import numpy as np
import pytest
import torch

import hyk
from hyk import adjoint, var, workloads as W

pytestmark = pytest.mark.gpu


def _loss_grad(sys_, x0, pars, tf, target):
    x = torch.tensor(x0, dtype=torch.float64, device="cuda", requires_grad=True)
    p = None if pars is None else torch.tensor(pars, dtype=torch.float64, device="cuda", requires_grad=True)
    xf, _ = adjoint.taylor_flow(sys_, x, tf, pars=p, tol=1e-15)
    loss = ((xf[:3] - torch.tensor(target, device="cuda")) ** 2).sum()
    loss.backward()
    return loss.item(), x.grad.cpu().numpy(), (None if p is None else p.grad.cpu().numpy())


def _loss(sys_, x0, pars, tf, target):
    with torch.no_grad():
        x = torch.tensor(x0, dtype=torch.float64, device="cuda")
        p = None if pars is None else torch.tensor(pars, dtype=torch.float64, device="cuda")
        xf, _ = adjoint.taylor_flow(sys_, x, tf, pars=p, tol=1e-15)
        return ((xf[:3].cpu().numpy() - target) ** 2).sum(axis=0)


def test_cr3bp_gradient_vs_finite_differences(libhyk):
    st, mu = W.cr3bp_ics(8, seed=31)
    rng = np.random.default_rng(3)
    target = st[:3] + rng.normal(0.0, 1e-2, st[:3].shape)
    tf = 12.0
    _, gx, gp = _loss_grad(W.cr3bp_sys(), st, mu, tf, target)
    for comp in range(6):
        d = 1e-6 * np.maximum(1.0, np.abs(st[comp]))
        a, b = st.copy(), st.copy()
        a[comp] += d
        b[comp] -= d
        fd = (_loss(W.cr3bp_sys(), a, mu, tf, target) - _loss(W.cr3bp_sys(), b, mu, tf, target)) / (2 * d)
        scale = np.maximum(np.abs(fd), 1e-3 * np.abs(gx).max())
        assert np.max(np.abs(gx[comp] - fd) / scale) < 1e-6, comp
    d = 1e-6 * mu
    fd = (_loss(W.cr3bp_sys(), st, mu + d, tf, target) - _loss(W.cr3bp_sys(), st, mu - d, tf, target)) / (2 * d[0])
    assert np.max(np.abs(gp[0] - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(gp).max())) < 1e-6


def test_cr3bp_gradient_vs_variational_equations(libhyk, oracle):
    st, mu = W.cr3bp_ics(4, seed=32)
    target = st[:3] + 1e-2
    tf = 12.0
    _, gx, gp = _loss_grad(W.cr3bp_sys(), st, mu, tf, target)
    vs = var.var_ode_sys(W.cr3bp_sys(), var.var_args.vars | var.var_args.params)
    full = np.concatenate([st, vs.initial_variational_state(4)])
    o = oracle.Oracle(vs.sys, full, pars=mu, order=19, mode=1)
    o.propagate_until(tf)
    xf = o.state[:6]
    J = o.state[6:].reshape(6, 7, 4)  # [component][arg][lane]
    g = np.zeros((6, 4))
    g[:3] = 2 * (xf[:3] - target)
    grad = np.einsum("ial,il->al", J, g)  # (7, lanes)
    rel_x = np.max(np.abs(grad[:6] - gx)) / np.max(np.abs(grad[:6]))
    rel_p = np.max(np.abs(grad[6] - gp[0])) / np.max(np.abs(grad[6]))
    assert rel_x < 1e-8 and rel_p < 1e-8


def test_every_operation_vs_finite_differences(libhyk):
    x, y = hyk.make_vars("x", "y")
    sys_ = [
        (x, hyk.exp(-y) * hyk.log(x) + hyk.sqrt(y) / x + hyk.cos(hyk.time) * hyk.par[1]),
        (y, hyk.par[0] / (x + 2.0) - x**-1.5 * hyk.par[1] + hyk.sin(x) * y),
    ]
    x0 = np.array([[1.1, 1.3, 0.9], [0.8, 0.6, 1.2]])
    pars = np.array([[0.3, 0.2, 0.4], [0.5, 0.7, 0.6]])
    target = np.zeros((2, 3))
    tf = 0.7

    def loss_np(xx, pp):
        with torch.no_grad():
            xf, _ = adjoint.taylor_flow(sys_, torch.tensor(xx, device="cuda"), tf,
                                        pars=torch.tensor(pp, device="cuda"), tol=1e-15)
            return (xf.cpu().numpy() ** 2).sum(axis=0)

    xt = torch.tensor(x0, device="cuda", requires_grad=True)
    pt = torch.tensor(pars, device="cuda", requires_grad=True)
    xf, _ = adjoint.taylor_flow(sys_, xt, tf, pars=pt, tol=1e-15)
    (xf**2).sum().backward()
    gx, gp = xt.grad.cpu().numpy(), pt.grad.cpu().numpy()
    del target
    for k, (arr, g) in enumerate(((x0, gx), (pars, gp))):
        for r in range(2):
            d = 1e-6
            a, b = arr.copy(), arr.copy()
            a[r] += d
            b[r] -= d
            if k == 0:
                fd = (loss_np(a, pars) - loss_np(b, pars)) / (2 * d)
            else:
                fd = (loss_np(x0, a) - loss_np(x0, b)) / (2 * d)
            assert np.max(np.abs(g[r] - fd) / np.maximum(np.abs(fd), 1e-8)) < 1e-6, (k, r)


def test_forward_matches_integrator(libhyk):
    st, mu = W.cr3bp_ics(64, seed=33)
    xf, _ = adjoint.taylor_flow(W.cr3bp_sys(), torch.tensor(st, device="cuda"), 5.0,
                                pars=torch.tensor(mu, device="cuda"), tol=1e-15)
    ta = hyk.taylor_adaptive_batch(W.cr3bp_sys(), st, pars=mu, tol=1e-15)
    ta.propagate_until(5.0)
    assert np.array_equal(xf.detach().cpu().numpy(), np.asarray(ta.state))


def test_cr3bp_gradient_vs_variational_equations_t50_256(libhyk, oracle):
    """The benchmark configuration's horizon: 256 seeded trajectories of the
    65536-trajectory CR3BP ensemble (mu per lane) to t = 50; the adjoint's
    gradient of loss = sum |r(50) - r*|^2 with respect to the initial state
    and mu against the first-order variational equations."""
    st, mu = W.cr3bp_ics(1 << 16, seed=3)
    idx = np.sort(np.random.default_rng(123).choice(1 << 16, 256, replace=False))
    st, mu = np.ascontiguousarray(st[:, idx]), np.ascontiguousarray(mu[:, idx])
    target = st[:3] + np.random.default_rng(3).normal(0.0, 1e-2, (3, 256))
    tf = 50.0
    _, gx, gp = _loss_grad(W.cr3bp_sys(), st, mu, tf, target)
    vs = var.var_ode_sys(W.cr3bp_sys(), var.var_args.vars | var.var_args.params)
    full = np.concatenate([st, vs.initial_variational_state(256)])
    o = oracle.Oracle(vs.sys, full, pars=mu, order=19, mode=1)
    o.propagate_until(tf)
    xf = o.state[:6]
    J = o.state[6:].reshape(6, 7, 256)
    g = np.zeros((6, 256))
    g[:3] = 2 * (xf[:3] - target)
    grad = np.einsum("ial,il->al", J, g)
    rel_x = np.max(np.abs(grad[:6] - gx), axis=0) / np.max(np.abs(grad[:6]), axis=0)
    rel_p = np.abs(grad[6] - gp[0]) / np.abs(grad[6])
    assert rel_x.max() < 1e-8 and rel_p.max() < 1e-8, (rel_x.max(), rel_p.max())


def test_longest_first_order_same_bits(libhyk):
    """The reverse sweep's lane order (longest tape first, or index order)
    changes the schedule only: the gradients are the same bits."""
    st, mu = W.cr3bp_ics(3000, seed=41)
    tf = np.exp(np.random.default_rng(5).uniform(0.0, np.log(20.0), 3000))
    grads = []
    for lpt in (True, False):
        adjoint.LONGEST_FIRST = lpt
        try:
            x = torch.tensor(st, device="cuda", requires_grad=True)
            p = torch.tensor(mu, device="cuda", requires_grad=True)
            xf, _ = adjoint.taylor_flow(W.cr3bp_sys(), x, torch.tensor(tf, device="cuda"), pars=p, tol=1e-15)
            (xf[:3] ** 2).sum().backward()
            grads.append((x.grad.cpu().numpy(), p.grad.cpu().numpy()))
        finally:
            adjoint.LONGEST_FIRST = True
    assert np.array_equal(grads[0][0], grads[1][0]) and np.array_equal(grads[0][1], grads[1][1])
    assert np.all(np.isfinite(grads[0][0]))
