"""Problem descriptions of the benchmark and parity workloads (seeded, synthetic).

Each workload mirrors an application's ``main.cc`` (fields, solve blocks, dependency strings)
and carries its initial condition evaluated at the support points in lattice order, the
nodal interpolation that ``SolverBase::set_initial_condition`` performs
(include/prismspf/solvers/solver_base.h:178-229).

  allen_cahn_2d       Allen-Cahn explicit, [0,100]^2, 128^2 cells Q1 (applications/allen_cahn/explicit)
  cahn_hilliard_3d    Cahn-Hilliard explicit, [0,64]^3, 64^3 cells Q2, periodic
                      (applications/cahn_hilliard/explicit)
  eshelby_3d          linear elasticity with eigenstrain of seeded inclusions
                      (applications/mechanics/eshelby_inclusion)
  coupled_acch_2d     coupled Allen-Cahn / Cahn-Hilliard (applications/coupled_allen_cahn_cahn_hilliard)
  allen_cahn_implicit_2d     Allen-Cahn with a Newton block (applications/allen_cahn/implicit)
  cahn_hilliard_implicit_2d  Cahn-Hilliard with a two-field Newton block (applications/cahn_hilliard/implicit)
"""
from __future__ import annotations

from dataclasses import dataclass, field as dfield

import numpy as np

from .problem import (Explicit, FieldAttributes, Linear, Newton, PostProcess, Primary, RectangularMesh, Scalar,
                      Secondary, SolveBlock, Vector, make_dependency_set)


def gauss_lobatto_points(n: int) -> np.ndarray:
    """Gauss-Lobatto points on [0,1] (endpoints and roots of P'_{n-1})."""
    if n == 2:
        return np.array([0.0, 1.0])
    inner = np.polynomial.legendre.Legendre.basis(n - 1).deriv().roots()
    t = np.concatenate([[-1.0], np.sort(inner.real), [1.0]])
    x = 0.5 * (t + 1.0)
    x = 0.5 * (x + (1.0 - x[::-1]))
    return x


def lattice_coordinates(mesh: RectangularMesh) -> np.ndarray:
    """Coordinates of the lattice nodes, shape (N, dim), index I + NX*(J + NY*K)."""
    gl = gauss_lobatto_points(mesh.degree + 1)
    axes = []
    for d in range(mesh.dim):
        nc = mesh.cells[d]
        h = mesh.size[d] / nc
        I = np.arange(mesh.degree * nc + 1)
        cell = np.minimum(I // mesh.degree, nc - 1)
        loc = I - cell * mesh.degree
        axes.append(mesh.lower[d] + (cell + gl[loc]) * h)
    grids = np.meshgrid(*axes, indexing="ij")
    # lattice order has x fastest: transpose to (z, y, x) before flattening
    return np.stack([g.transpose().ravel() for g in grids], axis=1)


@dataclass
class Workload:
    name: str
    mesh: RectangularMesh
    fields: list
    blocks: list
    model: str
    constants: list
    dt: float
    n_steps: int
    initial: dict = dfield(default_factory=dict)  # field index -> lattice-order vector
    seed: int = 0
    # mesh adaptivity: {min_level, max_level, period, criteria: [(field, flags, vlo, vhi, glo)]}
    # (flags 1 value, 2 gradient); None for a uniform mesh
    adaptivity: dict | None = None

    def make_problem(self):
        from .problem import Problem
        p = Problem(self.fields, self.blocks, self.mesh, self.model, self.constants, self.dt)
        if self.adaptivity is not None:
            p.set_adaptivity(self.adaptivity)
        for f, v in self.initial.items():
            p.upload(f, v)
        return p


def grain_field(x: np.ndarray, centres: np.ndarray, radii: np.ndarray, width: float) -> np.ndarray:
    r = np.sqrt(((x[:, None, :] - centres[None, :, :x.shape[1]]) ** 2).sum(-1))
    s = (0.5 * (1.0 - np.tanh((r - radii[None, :]) / width))).sum(1)
    return np.minimum(s, 1.0)


def allen_cahn_2d(refine: int = 7, degree: int = 1, seed: int = 1234, n_grains: int = 12, size: float = 100.0,
                  n_steps: int = 1000, dt: float = 0.01, m_well: float = 1.0, kappa: float = 2.0,
                  subdivisions=(1, 1)) -> Workload:
    """Allen-Cahn 2-D: fields n, mg_n, f_tot; blocks as applications/allen_cahn/explicit/main.cc."""
    mesh = RectangularMesh(dim=2, degree=degree, size=(size, size), subdivisions=tuple(subdivisions) + (1,),
                           global_refinement=refine)
    fields = [FieldAttributes("n", Scalar), FieldAttributes("mg_n", Scalar), FieldAttributes("f_tot", Scalar)]
    exp_block = SolveBlock(id=1, solve_type=Explicit, solve_timing=Primary, field_indices=[0],
                           dependencies_rhs=make_dependency_set(fields, {"old_1(n)", "grad(old_1(n))"}))
    pp_block = SolveBlock(id=2, solve_type=Explicit, solve_timing=PostProcess, field_indices=[1, 2],
                          dependencies_rhs=make_dependency_set(fields, {"n", "grad(n)"}))
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, size, size=(n_grains, 2))
    radii = rng.uniform(5.0, 15.0, size=n_grains)
    x = lattice_coordinates(mesh)
    n0 = grain_field(x, centres, radii, 2.0)
    return Workload("allen_cahn_2d", mesh, fields, [exp_block, pp_block], "allen_cahn", [m_well, kappa], dt,
                    n_steps, {0: n0}, seed)


def allen_cahn_amr_2d(refine: int = 4, degree: int = 2, min_level: int = 3, max_level: int = 6, period: int = 10,
                      seed: int = 1234, n_grains: int = 6, size: float = 100.0, n_steps: int = 100,
                      dt: float = 0.01) -> Workload:
    """Allen-Cahn 2-D on an adaptive mesh refined where 0.01 < n < 0.99 (the interfaces), as
    applications/allen_cahn/explicit with `mesh adaptivity = true` in its parameters."""
    wl = allen_cahn_2d(refine=refine, degree=degree, seed=seed, n_grains=n_grains, size=size, n_steps=n_steps, dt=dt)
    wl.name = "allen_cahn_amr_2d"
    wl.adaptivity = dict(min_level=min_level, max_level=max_level, period=period,
                         criteria=[(0, 1, 0.01, 0.99, 0.0)])
    return wl


def cahn_hilliard_amr(dim: int = 2, refine: int = 3, degree: int = 2, min_level: int = 2, max_level: int = 5,
                      period: int = 5, seed: int = 4321, size: float = 32.0, n_steps: int = 50,
                      dt: float = 1e-3, gradient_bound: float = 0.25) -> Workload:
    """Periodic Cahn-Hilliard on an adaptive mesh refined where the concentration gradient is
    large (a smooth two-phase initial field), fields c, mu, f_tot."""
    wl = cahn_hilliard_3d(refine=refine, degree=degree, seed=seed, size=size, n_steps=n_steps, dt=dt, dim=dim)
    x = lattice_coordinates(wl.mesh)
    rng = np.random.default_rng(seed)
    k = 2.0 * np.pi / size
    phase = rng.uniform(0.0, 2.0 * np.pi, size=2)
    c0 = 0.5 + 0.4 * np.tanh(4.0 * np.sin(k * x[:, 0] + phase[0]) * np.cos(k * x[:, 1] + phase[1]))
    wl.initial = {0: c0}
    wl.name = "cahn_hilliard_amr_%dd" % dim
    wl.adaptivity = dict(min_level=min_level, max_level=max_level, period=period,
                         criteria=[(0, 2, 0.0, 0.0, gradient_bound)])
    return wl


def cahn_hilliard_3d(refine: int = 6, degree: int = 2, seed: int = 4321, size: float = 64.0, n_steps: int = 200,
                     dt: float = 1e-4, McV: float = 1.0, KcV: float = 1.5, WcV: float = 4.0, dim: int = 3,
                     periodic: bool = True, subdivisions=(1, 1, 1)) -> Workload:
    """Cahn-Hilliard: fields c, mu, f_tot; blocks as applications/cahn_hilliard/explicit/main.cc.

    f = c^2 (1-c)^2 gives f' = 4 c (c-1)(c-1/2), i.e. the application's WcV = 4.
    """
    mesh = RectangularMesh(dim=dim, degree=degree, size=(size,) * dim + (1.0,) * (3 - dim),
                           subdivisions=tuple(subdivisions), global_refinement=refine,
                           periodic=(int(periodic),) * dim + (0,) * (3 - dim))
    fields = [FieldAttributes("c"), FieldAttributes("mu"), FieldAttributes("f_tot")]
    c_block = SolveBlock(id=0, solve_type=Explicit, solve_timing=Primary, field_indices=[0],
                         dependencies_rhs=make_dependency_set(fields, {"old_1(c)", "grad(old_1(mu))"}))
    mu_block = SolveBlock(id=1, solve_type=Explicit, solve_timing=Secondary, field_indices=[1],
                          dependencies_rhs=make_dependency_set(fields, {"c", "grad(c)"}))
    pp_block = SolveBlock(id=2, solve_type=Explicit, solve_timing=PostProcess, field_indices=[2],
                          dependencies_rhs=make_dependency_set(fields, {"c", "grad(c)"}))
    rng = np.random.default_rng(seed)
    N = int(np.prod(mesh.nodes))
    c0 = 0.5 + 0.05 * rng.uniform(-1.0, 1.0, size=N)
    return Workload("cahn_hilliard_%dd" % dim, mesh, fields, [c_block, mu_block, pp_block], "cahn_hilliard",
                    [McV, KcV, WcV], dt, n_steps, {0: c0}, seed)


def cubic_stiffness(C11: float, C12: float, C44: float) -> np.ndarray:
    C = np.zeros((6, 6))
    C[:3, :3] = C12
    np.fill_diagonal(C[:3, :3], C11)
    C[3, 3] = C[4, 4] = C[5, 5] = C44
    return C


def eshelby_3d(refine: int = 6, degree: int = 2, seed: int = 777, size: float = 64.0, n_incl: int = 40,
               dim: int = 3) -> Workload:
    """Elasticity with eigenstrain: field u (vector), block 1 Linear, u = 0 on boundary id 0."""
    mesh = RectangularMesh(dim=dim, degree=degree, size=(size,) * dim + (1.0,) * (3 - dim),
                           subdivisions=(1, 1, 1), global_refinement=refine)
    diri = {(c, 0): 0.0 for c in range(dim)}
    fields = [FieldAttributes("u", Vector, dirichlet=diri)]
    block = SolveBlock(id=1, solve_type=Linear, solve_timing=Secondary, field_indices=[0],
                       dependencies_rhs=make_dependency_set(fields, set()),
                       dependencies_lhs=make_dependency_set(fields, {"grad(lhs(u))"}))
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, size, size=(n_incl, 3))
    if dim == 2:
        centres[:, 2] = 0.0
    radii = rng.uniform(3.0, 6.0, size=n_incl)
    C = cubic_stiffness(250.0, 150.0, 100.0)
    consts = list(C.ravel()) + [0.01, 1.0, float(n_incl)]
    for i in range(n_incl):
        consts += [centres[i, 0], centres[i, 1], centres[i, 2], radii[i]]
    return Workload("eshelby_%dd" % dim, mesh, fields, [block], "eshelby", consts, 0.0, 1, {}, seed)


def coupled_acch_2d(refine: int = 8, degree: int = 2, seed: int = 99, size: float = 128.0, n_steps: int = 500,
                    dt: float = 2e-4, Mc: float = 1.0, Mn: float = 1.0, Kn: float = 2.0, n_precip: int = 8) -> Workload:
    """Coupled Allen-Cahn / Cahn-Hilliard: fields c, n, f_tot, mag_grad_c (coupled app main.cc).

    The application's free energy has f'' of about 10, so the explicit limit on the 256^2 Q2
    mesh of [0,128]^2 is about dt = 1e-3 / Mc; dt = 2e-4 keeps the step stable for the
    calibration targets (Mc up to 1.5)."""
    mesh = RectangularMesh(dim=2, degree=degree, size=(size, size), subdivisions=(1, 1, 1), global_refinement=refine)
    fields = [FieldAttributes("c"), FieldAttributes("n"), FieldAttributes("f_tot"), FieldAttributes("mag_grad_c")]
    exp_block = SolveBlock(id=0, solve_type=Explicit, solve_timing=Primary, field_indices=[0, 1],
                           dependencies_rhs=make_dependency_set(
                               fields, {"old_1(c)", "grad(old_1(c))", "old_1(n)", "grad(old_1(n))"}))
    pp_block = SolveBlock(id=1, solve_type=Explicit, solve_timing=PostProcess, field_indices=[2, 3],
                          dependencies_rhs=make_dependency_set(fields, {"n", "grad(n)", "c", "grad(c)"}))
    rng = np.random.default_rng(seed)
    x = lattice_coordinates(mesh)
    centres = rng.uniform(0.2 * size, 0.8 * size, size=(n_precip, 2))
    radii = rng.uniform(6.0, 14.0, size=n_precip)
    n0 = grain_field(x, centres, radii, 1.0)
    c0 = 0.009 + (0.125 - 0.009) * n0
    return Workload("coupled_acch_2d", mesh, fields, [exp_block, pp_block], "coupled_acch", [Mc, Mn, Kn], dt,
                    n_steps, {0: c0, 1: n0}, seed)


def allen_cahn_implicit_2d(refine: int = 5, degree: int = 1, seed: int = 1234, n_grains: int = 12, size: float = 100.0,
                           n_steps: int = 20, dt: float = 0.5, m_well: float = 1.0, kappa: float = 2.0) -> Workload:
    """Implicit Allen-Cahn: fields n, mg_n, f_tot; blocks as applications/allen_cahn/implicit/main.cc.

    Backward Euler through a Newton block (residual old_n - n - dt M f'(n), Jacobian
    1 + dt M f''(n) plus dt kappa M grad), so time steps far above the explicit limit work."""
    mesh = RectangularMesh(dim=2, degree=degree, size=(size, size), subdivisions=(1, 1, 1), global_refinement=refine)
    fields = [FieldAttributes("n", Scalar), FieldAttributes("mg_n", Scalar), FieldAttributes("f_tot", Scalar)]
    newton = SolveBlock(id=1, solve_type=Newton, solve_timing=Primary, field_indices=[0],
                        dependencies_rhs=make_dependency_set(fields, {"n", "grad(n)", "old_1(n)"}),
                        dependencies_lhs=make_dependency_set(fields, {"n", "change(n)", "grad(change(n))"}))
    pp_block = SolveBlock(id=2, solve_type=Explicit, solve_timing=PostProcess, field_indices=[1, 2],
                          dependencies_rhs=make_dependency_set(fields, {"n", "grad(n)"}))
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, size, size=(n_grains, 2))
    radii = rng.uniform(5.0, 15.0, size=n_grains)
    n0 = grain_field(lattice_coordinates(mesh), centres, radii, 2.0)
    return Workload("allen_cahn_implicit_2d", mesh, fields, [newton, pp_block], "allen_cahn_implicit",
                    [m_well, kappa], dt, n_steps, {0: n0}, seed)


def cahn_hilliard_implicit_2d(refine: int = 4, degree: int = 2, seed: int = 4321, size: float = 16.0,
                              n_steps: int = 10, dt: float = 0.01, McV: float = 1.0, KcV: float = 1.5,
                              WcV: float = 4.0) -> Workload:
    """Implicit Cahn-Hilliard: fields c, mu, f_tot; one Newton block over (c, mu) as
    applications/cahn_hilliard/implicit/main.cc (its Jacobian is not symmetric: BiCGStab)."""
    mesh = RectangularMesh(dim=2, degree=degree, size=(size, size), subdivisions=(1, 1, 1), global_refinement=refine)
    fields = [FieldAttributes("c"), FieldAttributes("mu"), FieldAttributes("f_tot")]
    newton = SolveBlock(id=0, solve_type=Newton, solve_timing=Primary, field_indices=[0, 1],
                        dependencies_rhs=make_dependency_set(fields, {"c", "grad(c)", "mu", "grad(mu)", "old_1(c)"}),
                        dependencies_lhs=make_dependency_set(fields, {"c", "grad(c)", "mu", "grad(mu)", "change(c)",
                                                                      "grad(change(c))", "change(mu)",
                                                                      "grad(change(mu))"}))
    pp_block = SolveBlock(id=2, solve_type=Explicit, solve_timing=PostProcess, field_indices=[2],
                          dependencies_rhs=make_dependency_set(fields, {"c", "grad(c)"}))
    rng = np.random.default_rng(seed)
    N = int(np.prod(mesh.nodes))
    c0 = 0.5 + 0.05 * rng.uniform(-1.0, 1.0, size=N)
    return Workload("cahn_hilliard_implicit_2d", mesh, fields, [newton, pp_block], "cahn_hilliard_implicit",
                    [McV, KcV, WcV], dt, n_steps, {0: c0, 1: np.zeros(N)}, seed)
