"""GPU tests of the hand-written adjoint of the coupled Allen-Cahn / Cahn-Hilliard explicit step.

* dot-product test against the tangent-linear model: <lambda_K, du_K> = <lambda_0, du_0> +
  dJ/dtheta . dtheta to 1e-10 relative (both linearisations share the pointwise Jacobians,
  so this pins the transposition of the sum-factorised apply);
* gradients against central finite differences of the loss J = sum_i m_i (c_K,i - t_i)^2
  through the forward path (ppf_run) within 1e-6 relative;
* the checkpoint budget changes the cost, not the gradient.
"""
import numpy as np
import pytest

from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_wl(**kw):
    args = dict(refine=3, degree=2, size=32.0, dt=1e-3, n_precip=3)
    args.update(kw)
    return W.coupled_acch_2d(**args)


def forward_final(wl, steps, Mc=None, Kn=None, n0=None):
    wl2 = W.coupled_acch_2d(refine=wl.mesh.global_refinement, degree=wl.mesh.degree, size=wl.mesh.size[0],
                            dt=wl.dt, Mc=wl.constants[0] if Mc is None else Mc, Mn=wl.constants[1],
                            Kn=wl.constants[2] if Kn is None else Kn, n_precip=3)
    wl2.initial = {0: wl.initial[0], 1: wl.initial[1] if n0 is None else n0}
    p = wl2.make_problem()
    p.solve(steps)
    c = p.download(0, age=1)
    mass = 1.0 / p.invm()
    p.close()
    return c, mass


def loss(c, target, mass):
    return float(np.sum(mass * (c - target) ** 2))


def test_adjoint_dot_product_with_tangent_linear(gpu_lib):
    wl = small_wl()
    K = 12
    p = wl.make_problem()
    N = p.n_nodes
    rng = np.random.default_rng(1)
    du0 = rng.normal(size=2 * N)
    dtheta = np.array([0.3, -0.7])
    duK = p.tangent_linear(0, K, du0, dtheta)
    lamK = rng.normal(size=2 * N)
    p.adjoint_forward(0, K, 4)
    dparams, lam0, _ = p.adjoint_backward(lamK)
    lhs = float(lamK @ duK)
    rhs = float(lam0 @ du0 + dparams @ dtheta)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs))


def test_adjoint_gradients_match_central_differences(gpu_lib):
    wl = small_wl()
    K = 20
    Mc, Mn, Kn = wl.constants
    target, mass = forward_final(wl, K, Mc=1.5 * Mc, Kn=0.5 * Kn)
    cK, _ = forward_final(wl, K)
    p = wl.make_problem()
    N = p.n_nodes
    p.adjoint_forward(0, K, 5)
    assert np.allclose(p.download(0), cK, rtol=0, atol=1e-13)
    dJ = np.concatenate([2.0 * mass * (cK - target), np.zeros(N)])
    dparams, du0, _ = p.adjoint_backward(dJ)
    for i, (name, val) in enumerate((("Mc", Mc), ("Kn", Kn))):
        eps = 1e-5 * val
        kp = {name: val + eps}
        km = {name: val - eps}
        jp = loss(forward_final(wl, K, **kp)[0], target, mass)
        jm = loss(forward_final(wl, K, **km)[0], target, mass)
        fd = (jp - jm) / (2 * eps)
        assert abs(dparams[i] - fd) <= 1e-6 * abs(fd), (name, dparams[i], fd)
    # initial n along a smooth direction
    x = W.lattice_coordinates(wl.mesh)
    d = np.sin(2 * np.pi * x[:, 0] / wl.mesh.size[0]) * np.cos(2 * np.pi * x[:, 1] / wl.mesh.size[1])
    eps = 1e-6
    n0 = wl.initial[1]
    jp = loss(forward_final(wl, K, n0=n0 + eps * d)[0], target, mass)
    jm = loss(forward_final(wl, K, n0=n0 - eps * d)[0], target, mass)
    fd = (jp - jm) / (2 * eps)
    adj = float(du0[N:] @ d)
    assert abs(adj - fd) <= 1e-6 * abs(fd), (adj, fd)


def test_checkpoint_budget_does_not_change_gradients(gpu_lib):
    wl = small_wl()
    K = 16
    p = wl.make_problem()
    N = p.n_nodes
    rng = np.random.default_rng(4)
    lamK = rng.normal(size=2 * N)
    results = []
    for slots in (2, 5, K + 1):
        p.upload(0, wl.initial[0])
        p.upload(1, wl.initial[1])
        p.adjoint_forward(0, K, slots)
        dparams, lam0, steps = p.adjoint_backward(lamK)
        results.append((dparams, lam0, steps))
    for dparams, lam0, _ in results[1:]:
        assert np.allclose(dparams, results[0][0], rtol=1e-12, atol=0)
        assert np.linalg.norm(lam0 - results[0][1]) <= 1e-12 * np.linalg.norm(results[0][1])
    assert results[0][2] > results[1][2] > results[2][2] == K
