"""CPU tests of the oracle (the CPU restatement) against known answers.

The reference's own tests hold no golden vectors for the operator path, so the oracle is
pinned by closed forms: Gauss-Lobatto rules, deal.II's documented FE_Q dof layout on a
single cell, conservation laws, discrete-Laplacian eigenpairs and the elasticity patch test.
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import workloads as W
from phasefield_gb300.problem import FieldAttributes, RectangularMesh, SolveBlock, Vector, Linear, make_dependency_set


@pytest.mark.parametrize("n,x,w", [
    (2, [0, 1], [1 / 2, 1 / 2]),
    (3, [0, 0.5, 1], [1 / 6, 2 / 3, 1 / 6]),
    (4, [0, (1 - 1 / math.sqrt(5)) / 2, (1 + 1 / math.sqrt(5)) / 2, 1], [1 / 12, 5 / 12, 5 / 12, 1 / 12]),
    (5, [0, (1 - math.sqrt(3 / 7)) / 2, 0.5, (1 + math.sqrt(3 / 7)) / 2, 1],
     [1 / 20, 49 / 180, 16 / 45, 49 / 180, 1 / 20]),
])
def test_gauss_lobatto_rules(n, x, w):
    ox, ow, D = po.gl_rule(n)
    assert np.allclose(ox, x, atol=1e-15, rtol=0)
    assert np.allclose(ow, w, atol=1e-15, rtol=0)
    # derivative matrix differentiates polynomials of degree n-1 exactly
    for p in range(n):
        assert np.allclose(D @ ox ** p, p * ox ** max(p - 1, 0) if p else 0.0, atol=1e-12)


def test_gl3_derivative_matrix():
    _, _, D = po.gl_rule(3)
    assert np.allclose(D, [[-3, 4, -1], [-1, 0, 1], [1, -4, 3]], atol=1e-14)


def _mesh_wl(dim, degree, refine=0, subdivisions=(1, 1, 1), periodic=(0, 0, 0), vector=False):
    wl = W.allen_cahn_2d(refine=refine, degree=degree) if dim == 2 and not vector else None
    if wl is None or vector:
        mesh = RectangularMesh(dim=dim, degree=degree, size=(1.0,) * 3, subdivisions=subdivisions,
                               global_refinement=refine, periodic=periodic)
        fields = [FieldAttributes("u", Vector if vector else 0)]
        blk = SolveBlock(id=1, solve_type=Linear, field_indices=[0],
                         dependencies_lhs=make_dependency_set(fields, {"grad(lhs(u))"}))
        consts = list(np.eye(6).ravel()) + [0.0, 1.0, 0.0]
        wl = W.Workload("t", mesh, fields, [blk], "eshelby", consts, 0.0, 0, {})
    return wl


def test_dealii_numbering_single_q2_cell():
    # FE_Q(2) on one quad: vertices, then lines x=0, x=1, y=0, y=1, then the interior
    wl = W.allen_cahn_2d(refine=0, degree=2)
    o = po.Oracle(wl)
    L = o.lattice(0)[:, :2]
    assert L.tolist() == [[0, 0], [2, 0], [0, 2], [2, 2], [0, 1], [2, 1], [1, 0], [1, 2], [1, 1]]


def test_dealii_numbering_two_q1_cells():
    wl = W.allen_cahn_2d(refine=0, degree=1, subdivisions=(2, 1))
    wl.mesh.size = (2.0, 1.0)
    o = po.Oracle(wl)
    L = o.lattice(0)[:, :2]
    assert L.tolist() == [[0, 0], [1, 0], [0, 1], [1, 1], [2, 0], [2, 1]]


def test_dealii_numbering_refined_child_order():
    # one refinement of a single Q1 cell: children in lexicographic order, first-touch dofs
    wl = W.allen_cahn_2d(refine=1, degree=1)
    o = po.Oracle(wl)
    L = o.lattice(0)[:, :2].tolist()
    assert L[:4] == [[0, 0], [1, 0], [0, 1], [1, 1]]  # child 0
    assert L[4:6] == [[2, 0], [2, 1]]                  # child 1 adds its right vertices
    assert L[6:8] == [[0, 2], [1, 2]]                  # child 2 adds its top vertices
    assert L[8:] == [[2, 2]]                           # child 3


def test_vector_numbering_is_component_major_per_object():
    wl = _mesh_wl(2, 2, vector=True)
    o = po.Oracle(wl)
    L = o.lattice(1)
    # first vertex carries components 0 and 1 consecutively (one dof per vertex per component)
    assert L[0].tolist()[:2] == [0, 0] and L[0, 3] == 0
    assert L[1].tolist()[:2] == [0, 0] and L[1, 3] == 1
    assert o.n_dofs(1) == 2 * o.n_dofs(0)


@pytest.mark.parametrize("dim,degree", [(2, 1), (2, 2), (2, 3), (2, 4), (3, 1), (3, 2)])
def test_lumped_mass_sums_to_volume(dim, degree):
    wl = W.cahn_hilliard_3d(refine=2 if dim == 3 else 3, degree=degree, dim=dim, size=3.0, periodic=True)
    o = po.Oracle(wl)
    im = o.invm(0)
    mass = np.where(im > 0, 1.0 / np.where(im > 0, im, 1.0), 0.0)
    assert abs(mass.sum() - 3.0 ** dim) < 1e-11 * 3.0 ** dim
    # periodic images carry no mass of their own
    nn = wl.mesh.nodes
    img = mass.reshape(nn[::-1])
    assert np.all(img[..., -1] == 0)


@pytest.mark.parametrize("value", [0.0, 1.0])
def test_allen_cahn_constant_fixed_points(value):
    wl = W.allen_cahn_2d(refine=3, degree=2)
    wl.initial = {0: np.full(int(np.prod(wl.mesh.nodes)), value)}
    o = po.Oracle(wl)
    assert o.run(5) == 0
    assert np.max(np.abs(o.get(0, 1) - value)) < 1e-14


def test_cahn_hilliard_mass_conservation():
    wl = W.cahn_hilliard_3d(refine=2, degree=2, n_steps=10, dt=1e-3)
    o = po.Oracle(wl)
    im = o.invm(0)
    jxw = np.where(im > 0, 1.0 / np.where(im > 0, im, 1.0), 0.0)
    o.run(1)  # the first step reads the non-distributed initial condition
    m1 = (jxw * o.get(0, 1)).sum()
    o.run(15)
    m2 = (jxw * o.get(0, 1)).sum()
    assert abs(m2 - m1) < 1e-13 * abs(m1)


@pytest.mark.parametrize("m", [1, 3])
def test_periodic_q1_laplacian_eigenvector(m):
    # mu block with WcV = 0: mu = KcV * invM K c; for c = cos(2 pi m x / L) on a periodic Q1
    # mesh the lumped discrete Laplacian has eigenvalue (2/h^2)(1 - cos(2 pi m h / L))
    L_ = 8.0
    wl = W.cahn_hilliard_3d(refine=4, degree=1, dim=2, size=L_, WcV=0.0, KcV=1.0, periodic=True)
    o = po.Oracle(wl)
    x = W.lattice_coordinates(wl.mesh)
    c = np.cos(2 * np.pi * m * x[:, 0] / L_)
    o.set(0, c)
    mu = o.apply(1, 0, None, scale=1)
    h = L_ / wl.mesh.cells[0]
    lam = 2.0 / h ** 2 * (1.0 - math.cos(2 * math.pi * m * h / L_))
    nn = wl.mesh.nodes
    mask = np.ones(nn[::-1], bool)
    mask[-1, :] = False
    mask[:, -1] = False
    assert np.allclose(mu[mask.ravel()], lam * c[mask.ravel()], rtol=0, atol=1e-12)


def test_elasticity_patch_uniform_eigenstrain():
    # uniform eigenstrain e0*I, no Dirichlet rows: u = e0 * x is stress-free, so
    # A u - b = 0 at every dof (A: compute_lhs, b = -compute_rhs contribution)
    mesh = RectangularMesh(dim=3, degree=2, size=(4.0, 4.0, 4.0), global_refinement=1)
    fields = [FieldAttributes("u", Vector)]
    blk = SolveBlock(id=1, solve_type=Linear, field_indices=[0],
                     dependencies_rhs=make_dependency_set(fields, set()),
                     dependencies_lhs=make_dependency_set(fields, {"grad(lhs(u))"}))
    C = W.cubic_stiffness(250.0, 150.0, 100.0)
    e0 = 0.01
    consts = list(C.ravel()) + [e0, 1.0, 1.0, 2.0, 2.0, 2.0, 1e6]
    wl = W.Workload("patch", mesh, fields, [blk], "eshelby", consts, 0.0, 0, {})
    o = po.Oracle(wl)
    x = W.lattice_coordinates(mesh)
    u = np.concatenate([e0 * x[:, 0], e0 * x[:, 1], e0 * x[:, 2]])
    Au = o.apply(0, 1, u)
    rhs = o.apply(0, 0, None)
    assert np.max(np.abs(Au + rhs)) < 1e-12 * np.max(np.abs(Au))
    assert np.max(np.abs(Au)) > 1e-3


@pytest.mark.parametrize("preconditioner,depth", [(1, 1), (2, 2), (2, 3)])
def test_preconditioned_solves_agree_with_plain_cg(preconditioner, depth):
    wl = W.eshelby_3d(refine=2, degree=2, size=8.0, n_incl=3)
    base = dict(tolerance_type=1, tolerance=1e-11, max_iterations=3000, smoother_degree=4)
    o0 = po.Oracle(wl)
    o0.set_linear_params(0, preconditioner=0, **base)
    rc0, its0, _ = o0.linear_solve(0)
    o1 = po.Oracle(wl)
    o1.set_linear_params(0, preconditioner=preconditioner, mg_depth=depth, **base)
    rc1, its1, res1 = o1.linear_solve(0)
    assert rc0 == 0 and rc1 == 0
    assert res1 < 1e-11
    assert its1 < its0
    u0, u1 = o0.get(0), o1.get(0)
    assert np.linalg.norm(u1 - u0) < 1e-8 * np.linalg.norm(u0)


def test_gmg_iterations_fall_with_depth_symmetric_scaling():
    wl = W.eshelby_3d(refine=3, degree=1, size=16.0, n_incl=5)
    its = []
    for depth in (1, 2, 3):
        o = po.Oracle(wl)
        o.set_linear_params(0, tolerance_type=0, tolerance=1e-9, max_iterations=800, preconditioner=2, mg_depth=depth,
                            smoother_degree=4)
        rc, it, _ = o.linear_solve(0)
        assert rc == 0
        its.append(it)
    assert its[0] > its[1] > its[2]


# ---------------------------------------------------------------------------------------------
# Newton solves (newton_solver.h:73-156)
# ---------------------------------------------------------------------------------------------
def _implicit_ac(dt=2.0, refine=4):
    wl = W.allen_cahn_implicit_2d(refine=refine, dt=dt)
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=1, tolerance=1e-12, max_iterations=2000)
    o.set_newton_params(0, max_iterations=50, tolerance=1e-10)
    return wl, o


def test_newton_allen_cahn_converges_and_is_bounded_at_large_dt():
    # dt = 2 is 30x the explicit limit of this mesh; backward Euler stays within [0, 1]
    wl, o = _implicit_ac(dt=2.0)
    assert o.run(6, 6) == 0
    n = o.get(0, 1)
    assert np.all(n > -1e-3) and np.all(n < 1.0 + 1e-3)
    rc, its, lin, res = o.newton_solve(0)
    assert rc == 0 and its <= 6 and res < 1e-10


def test_newton_allen_cahn_fixed_points():
    wl, o = _implicit_ac(dt=5.0, refine=3)
    for value in (0.0, 1.0):
        v = np.full(o.n_dofs(0), value)
        o.set(0, v, age=1)
        o.set(0, v, age=0)
        rc, its, lin, res = o.newton_solve(0)
        assert rc == 0 and its == 0  # the residual of a fixed point is already zero
        assert np.allclose(o.get(0, 0), value, atol=1e-14)


def test_newton_cg_and_bicgstab_agree_on_a_symmetric_jacobian():
    sols = []
    for solver in (0, 1):
        wl, o = _implicit_ac(dt=1.0)
        o.set_linear_params(0, tolerance_type=1, tolerance=1e-13, max_iterations=2000, solver_type=solver)
        o.set(0, wl.initial[0], age=1)
        o.set(0, wl.initial[0], age=0)
        rc, its, lin, res = o.newton_solve(0)
        assert rc == 0
        sols.append(o.get(0, 0))
    assert np.linalg.norm(sols[0] - sols[1]) / np.linalg.norm(sols[1]) < 1e-10


def test_newton_cahn_hilliard_two_field_block_conserves_mass():
    wl = W.cahn_hilliard_implicit_2d(refine=3, dt=0.05)
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=1, tolerance=1e-13, max_iterations=4000, solver_type=1)
    o.set_newton_params(0, max_iterations=50, tolerance=1e-11)
    assert o.run(4) == 0
    m = o.invm(0)
    mass = np.where(m > 0, 1.0 / np.where(m > 0, m, 1.0), 0.0)
    assert abs((mass * o.get(0, 1)).sum() - (mass * wl.initial[0]).sum()) < 1e-10 * (mass * wl.initial[0]).sum()
    # the step is not the identity: the interface has moved
    assert np.linalg.norm(o.get(0, 1) - wl.initial[0]) > 1e-4
