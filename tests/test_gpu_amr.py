"""Adaptive meshes on the GPU against the oracle (oracle/oracle.cc, adaptive-mesh section): the
same active cells in the same order, the same DoF numbering, hanging-node lines and lumped mass,
and the same fields after increments that remesh (RefinementManager,
src/core/refinement_manager.cc:42-439)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NATIVE = capi.ORDER_NATIVE


def _ac(degree, **kw):
    return W.allen_cahn_amr_2d(refine=3, degree=degree, min_level=2, max_level=5 if degree == 2 else 6, **kw)


def _ac_dirichlet():
    wl = _ac(2)
    wl.fields[0].dirichlet = {(0, 0): 1.0, (0, 3): 0.25}
    return wl


CASES = [
    ("ac2_q2", lambda: _ac(2)),
    ("ac2_q1", lambda: _ac(1)),
    ("ac2_q2_dirichlet", _ac_dirichlet),
    ("ch2_q2_periodic", lambda: W.cahn_hilliard_amr(2)),
    ("ch3_q1_periodic", lambda: W.cahn_hilliard_amr(3, refine=2, degree=1, max_level=4, size=16.0,
                                                     gradient_bound=0.1)),
]


def _pair(make):
    wl = make()
    return wl, wl.make_problem(), po.Oracle(wl, adaptivity=wl.adaptivity)


def _same_mesh(p, o):
    assert np.array_equal(p.cells(), o.cells())
    assert p.n_nodes == o.n_nodes()
    assert np.array_equal(p.cell_dofs().astype(np.int64), o.cell_dofs(0))
    assert np.array_equal(p.node_points(), o.node_points())
    pc, pm, pw = p.hanging()
    oc, om, ow = o.hanging()
    assert np.array_equal(pc, oc) and np.array_equal(pm.astype(np.int64), om) and np.array_equal(pw, ow)


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_initial_refinement_matches_the_oracle(name, make):
    wl, p, o = _pair(make)
    p.solve(0)
    assert o.run(0, 0) == 0
    assert p.mesh_version > 0
    assert len(np.unique(p.cells()[:, 0])) > 1
    _same_mesh(p, o)
    ref = o.invm_native(0)
    assert np.abs(p.invm() - ref).max() <= 1e-14 * np.abs(ref).max()
    for f in range(len(wl.fields)):
        a = p.download(f, 1 if f == 0 else 0, NATIVE)
        b = o.get_native(f, 1 if f == 0 else 0)
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max()), f


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_increments_with_remeshing_match_the_oracle(name, make):
    wl, p, o = _pair(make)
    n = 12
    p.solve(n)
    assert o.run(n, 0) == 0
    _same_mesh(p, o)
    for f, blk in enumerate(wl.fields):
        age = 1 if f == 0 else 0
        a = p.download(f, age, NATIVE)
        b = o.get_native(f, age)
        assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max()), f


def test_lattice_io_on_the_initial_mesh_round_trips():
    wl = W.cahn_hilliard_amr(2)
    p = wl.make_problem()
    v = wl.initial[0]
    back = p.download(0, 0)
    # periodic images read their master, which holds the image's value for a periodic field
    assert np.abs(back - v).max() < 0.5
    x = W.lattice_coordinates(wl.mesh)
    inner = (x[:, 0] < wl.mesh.size[0]) & (x[:, 1] < wl.mesh.size[1])
    assert np.array_equal(back[inner], v[inner])


def test_apply_constraints_interpolates_hanging_nodes():
    wl, p, o = _pair(lambda: _ac(2))
    p.solve(0)
    x = p.node_points()
    L = wl.mesh.size[0]
    q = 1.0 + x[:, 0] / L - 0.5 * (x[:, 1] / L) ** 2 + 0.25 * x[:, 0] * x[:, 1] / L ** 2
    cnt, _, _ = p.hanging()
    noisy = q.copy()
    noisy[cnt > 0] = 7.0
    p.upload(1, noisy, 0, NATIVE)
    p.apply_constraints(1)
    assert np.abs(p.download(1, 0, NATIVE) - q).max() < 1e-13


def _solver_pair(wl, lin, newton=None):
    p = wl.make_problem()
    o = po.Oracle(wl, adaptivity=wl.adaptivity)
    for b, blk in enumerate(wl.blocks):
        if blk.solve_type in (2, 3):  # Linear, Newton
            p.set_linear_params(b, **lin)
            o.set_linear_params(b, **lin)
            if newton:
                p.set_newton_params(b, **newton)
                o.set_newton_params(b, **newton)
    return p, o


def _rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_newton_allen_cahn_on_an_adaptive_mesh_matches_the_oracle():
    wl = W.allen_cahn_implicit_2d(refine=4, dt=1.0)
    wl.adaptivity = dict(min_level=3, max_level=6, period=2, criteria=[(0, 1, 0.01, 0.99, 0.0)])
    p, o = _solver_pair(wl, dict(tolerance_type=1, tolerance=1e-12, max_iterations=3000),
                        dict(max_iterations=50, tolerance=1e-10))
    n = 5
    p.solve(n, output_every=n)
    assert o.run(n, n) == 0
    _same_mesh(p, o)
    assert len(np.unique(p.cells()[:, 0])) > 1
    for f, age in ((0, 1), (1, 0), (2, 0)):
        assert _rel_l2(p.download(f, age, NATIVE), o.get_native(f, age)) < 1e-8, f


def test_newton_cahn_hilliard_bicgstab_on_an_adaptive_mesh_matches_the_oracle():
    wl = W.cahn_hilliard_implicit_2d(refine=3, dt=0.05)
    wl.adaptivity = dict(min_level=2, max_level=4, period=2, criteria=[(0, 2, 0.0, 0.0, 0.025)])
    p, o = _solver_pair(wl, dict(tolerance_type=1, tolerance=1e-13, max_iterations=4000, solver_type=1),
                        dict(max_iterations=50, tolerance=1e-11))
    n = 4
    p.solve(n)
    assert o.run(n) == 0
    _same_mesh(p, o)
    assert len(np.unique(p.cells()[:, 0])) > 1
    assert _rel_l2(p.download(0, 1, NATIVE), o.get_native(0, 1)) < 1e-8
    assert _rel_l2(p.download(1, 0, NATIVE), o.get_native(1, 0)) < 1e-8


def test_linear_elasticity_on_an_adaptive_mesh_matches_the_oracle():
    """A Linear block (vector field, CG without preconditioner) on a graded mesh with an
    inhomogeneous Dirichlet face, so hanging nodes meet Dirichlet nodes in the lift."""
    wl = W.eshelby_3d(refine=2, degree=2, size=16.0, n_incl=5, dim=3)
    wl.fields[0].dirichlet = {(0, 0): 0.01, (1, 0): 0.0, (2, 0): 0.0}
    wl.adaptivity = dict(min_level=1, max_level=3, period=1, criteria=[(0, 2, 0.02, 1e9, 0.0)])
    p, o = _solver_pair(wl, dict(tolerance_type=1, tolerance=1e-11, max_iterations=5000))
    p.solve(1)
    assert o.run(1, 0) == 0
    _same_mesh(p, o)
    assert len(np.unique(p.cells()[:, 0])) > 1
    assert (p.hanging()[0] > 0).any()
    assert _rel_l2(p.download(0, 0, NATIVE), o.get_native(0, 0)) < 1e-8


def test_dirichlet_function_values_on_every_mesh():
    """ppf_set_dirichlet_function: the engine evaluates the callback at the Dirichlet nodes of
    every mesh it builds. A callback returning the per-face constants reproduces the constant
    run; a position-dependent one leaves its values on the Dirichlet nodes after
    remeshing increments."""
    import ctypes as C

    def make():
        wl = _ac(2)
        wl.fields[0].dirichlet = {(0, 0): 1.0, (0, 3): 0.25}
        return wl

    ref = make().make_problem()
    ref.solve(6)
    consts = {0: 1.0, 3: 0.25}
    calls = []

    @capi.DIRICHLET_FN
    def const_fn(user, field, comp, bid, x, t):
        calls.append(bid)
        return consts[bid]

    p = make().make_problem()
    assert p.lib.ppf_set_dirichlet_function(p.h, 0, const_fn, None) == capi.PPF_OK
    p.solve(6)
    assert calls and set(calls) <= {0, 3}
    assert np.array_equal(p.cells(), ref.cells())
    # the same run up to the summation order of the scatter's atomics
    assert np.abs(p.download(0, 1, NATIVE) - ref.download(0, 1, NATIVE)).max() < 1e-13

    @capi.DIRICHLET_FN
    def ramp(user, field, comp, bid, x, t):
        return 0.5 + 0.004 * x[1] if bid == 0 else 0.1 + 0.002 * x[0]

    q = make().make_problem()
    assert q.lib.ppf_set_dirichlet_function(q.h, 0, ramp, None) == capi.PPF_OK
    q.solve(6)
    assert q.mesh_version > 0
    x = q.node_points()
    cmap = q.constraint_map(0)
    cnt, _, _ = q.hanging()
    u = q.download(0, 1, NATIVE)
    L = 100.0
    on0 = np.isclose(x[:, 0], 0.0) & (cmap < 0)
    on3 = np.isclose(x[:, 1], L) & (cmap < 0) & ~np.isclose(x[:, 0], 0.0)
    assert on0.sum() > 0 and on3.sum() > 0
    assert np.abs(u[on0] - (0.5 + 0.004 * x[on0, 1])).max() < 1e-15
    assert np.abs(u[on3] - (0.1 + 0.002 * x[on3, 0])).max() < 1e-15
    # hanging boundary nodes interpolate the (linear) boundary values of their coarse face
    hb = (cnt > 0) & np.isclose(x[:, 0], 0.0)
    if hb.any():
        assert np.abs(u[hb] - (0.5 + 0.004 * x[hb, 1])).max() < 1e-14
