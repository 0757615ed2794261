"""GPU tests of the linear-solve path (LinearSolver + GMG) against the oracle.

Bars: operator diagonal within 1e-12 relative L2 (same probes, same scaling); solutions of
CG / Chebyshev-CG / GMG-CG within 1e-8 relative L2 of the oracle's (both stop at an absolute
residual of 1e-10 of the scaled system); iteration counts equal within 10 %; the mixed-precision
V-cycle reaches the same tolerance and the same solution within 1e-8.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def small_elasticity(degree=2, refine=3, dim=3):
    return W.eshelby_3d(refine=refine, degree=degree, size=16.0, n_incl=5, dim=dim)


@pytest.mark.parametrize("tolerance_type", [0, 1])
@pytest.mark.parametrize("degree", [1, 2])
def test_lhs_diagonal_matches_oracle(gpu_lib, degree, tolerance_type):
    wl = small_elasticity(degree=degree, refine=2)
    p = wl.make_problem()
    p.set_linear_params(0, tolerance_type=tolerance_type)
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=tolerance_type)
    assert rel_l2(p.lhs_diagonal(0), o.diagonal(0)) < 1e-12


@pytest.mark.parametrize("preconditioner,depth", [(0, 1), (1, 1), (2, 2), (2, 3)])
def test_linear_solve_matches_oracle(gpu_lib, preconditioner, depth):
    wl = small_elasticity(degree=2, refine=3)
    prm = dict(tolerance_type=1, tolerance=1e-10, max_iterations=1500, preconditioner=preconditioner, mg_depth=depth,
               smoother_degree=4)
    p = wl.make_problem()
    p.set_linear_params(0, **prm)
    its, res = p.linear_solve(0)
    o = po.Oracle(wl)
    o.set_linear_params(0, **prm)
    rc, oits, ores = o.linear_solve(0)
    assert rc == 0
    assert res < 1e-10
    assert abs(its - oits) <= max(2, 0.1 * oits)
    assert rel_l2(p.download(0), o.get(0)) < 1e-8


@pytest.mark.parametrize("degree", [1, 2])
def test_mixed_precision_gmg_reaches_fp64_solution(gpu_lib, degree):
    wl = small_elasticity(degree=degree, refine=3)
    prm = dict(tolerance_type=1, tolerance=1e-10, max_iterations=1500, preconditioner=2, mg_depth=3, smoother_degree=4)
    p64 = wl.make_problem()
    p64.set_linear_params(0, **prm)
    its64, _ = p64.linear_solve(0)
    pmx = wl.make_problem()
    pmx.set_linear_params(0, mixed_precision=1, **prm)
    itsmx, resmx = pmx.linear_solve(0)
    assert resmx < 1e-10
    assert itsmx <= 1.5 * its64 + 2
    assert rel_l2(pmx.download(0), p64.download(0)) < 1e-8


def test_linear_block_runs_in_increment_loop(gpu_lib):
    wl = small_elasticity(degree=1, refine=2)
    p = wl.make_problem()
    p.set_linear_params(0, tolerance_type=1, tolerance=1e-10, max_iterations=1000, preconditioner=2, mg_depth=2,
                        smoother_degree=4)
    p.solve(0)  # increment 0 solves Secondary (Uninitialized) linear blocks
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=1, tolerance=1e-10, max_iterations=1000, preconditioner=2, mg_depth=2,
                        smoother_degree=4)
    assert o.run(0) == 0
    assert rel_l2(p.download(0), o.get(0)) < 1e-8


@pytest.mark.parametrize("tolerance_type", [0])
def test_inhomogeneous_dirichlet_lift_matches_oracle(gpu_lib, tolerance_type):
    # u = 0 on x = 0 and a prescribed displacement u_x = 0.05 on x = 16 (boundary id 1):
    # rhs -= S A_plain g (linear_solver.h:316-327), then x = x_hom + g. With the one-sided
    # invM^1/2 scaling (RMSEPerField) CG on S A stagnates near 3e-6 for this lift in the oracle
    # and on the GPU alike, so the lift is compared on the unscaled system.
    wl = small_elasticity(degree=2, refine=2)
    wl.fields[0].dirichlet[(0, 1)] = 0.05
    prm = dict(tolerance_type=tolerance_type, tolerance=1e-11, max_iterations=2000, preconditioner=2, mg_depth=2,
               smoother_degree=4)
    p = wl.make_problem()
    p.set_linear_params(0, **prm)
    p.linear_solve(0)
    o = po.Oracle(wl)
    o.set_linear_params(0, **prm)
    rc, _, _ = o.linear_solve(0)
    assert rc == 0
    u, ref = p.download(0), o.get(0)
    assert rel_l2(u, ref) < 1e-8
    # the prescribed face carries the Dirichlet value
    x = W.lattice_coordinates(wl.mesh)
    face = np.isclose(x[:, 0], 16.0)
    assert np.allclose(u[: len(x)][face], 0.05, rtol=0, atol=1e-14)


def test_nonconvergence_reports_noconv(gpu_lib):
    wl = small_elasticity(degree=1, refine=2)
    p = wl.make_problem()
    p.set_linear_params(0, tolerance_type=1, tolerance=1e-14, max_iterations=3, preconditioner=0)
    with pytest.raises(capi.PPFError) as e:
        p.linear_solve(0)
    assert e.value.code == capi.PPF_ERR_NOCONV
