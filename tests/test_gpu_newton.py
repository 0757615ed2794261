"""GPU tests of Newton blocks (NewtonSolver::solve_impl, newton_solver.h:73-156) against the oracle.

Both sides run the same Newton loop (start from old_1, constraints, scaled residual, Krylov
solve warm-started from the previous change, update) with the same Krylov method. Their
reductions round differently, so the iterates agree to the solver tolerances, not bitwise.
Bars: fields within 1e-8 relative L2 after several implicit increments (Newton tolerance 1e-10,
Krylov tolerance 1e-12); Newton iteration counts equal.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _both(wl, lin, newton):
    p = wl.make_problem()
    p.set_linear_params(0, **lin)
    p.set_newton_params(0, **newton)
    o = po.Oracle(wl)
    o.set_linear_params(0, **lin)
    o.set_newton_params(0, **newton)
    return p, o


@pytest.mark.parametrize("preconditioner", [0, 1])
def test_newton_allen_cahn_matches_oracle(gpu_lib, preconditioner):
    wl = W.allen_cahn_implicit_2d(refine=4, dt=1.0)
    lin = dict(tolerance_type=1, tolerance=1e-12, max_iterations=3000, preconditioner=preconditioner,
               smoother_degree=4)
    p, o = _both(wl, lin, dict(max_iterations=50, tolerance=1e-10))
    n = 5
    p.solve(n, output_every=n)
    assert o.run(n, n) == 0
    assert rel_l2(p.download(0, age=1), o.get(0, 1)) < 1e-8
    for f in (1, 2):
        assert rel_l2(p.download(f), o.get(f, 0)) < 1e-8, f
    # one more solve from the same state: same Newton iteration count, converged residual
    its, lin_its, res = p.newton_solve(0)
    rc, oits, olin, ores = o.newton_solve(0)
    assert rc == 0 and its == oits and res < 1e-10


def test_newton_cahn_hilliard_bicgstab_matches_oracle(gpu_lib):
    wl = W.cahn_hilliard_implicit_2d(refine=3, dt=0.05)
    lin = dict(tolerance_type=1, tolerance=1e-13, max_iterations=4000, solver_type=1)
    p, o = _both(wl, lin, dict(max_iterations=50, tolerance=1e-11))
    n = 4
    p.solve(n)
    assert o.run(n) == 0
    assert rel_l2(p.download(0, age=1), o.get(0, 1)) < 1e-8
    assert rel_l2(p.download(1), o.get(1, 0)) < 1e-8
    # mass of c is conserved by the implicit step
    m = o.invm(0)
    mass = np.where(m > 0, 1.0 / np.where(m > 0, m, 1.0), 0.0)
    c = p.download(0, age=1)
    assert abs((mass * c).sum() - (mass * wl.initial[0]).sum()) < 1e-10 * (mass * wl.initial[0]).sum()


def test_newton_reports_noconv(gpu_lib):
    wl = W.allen_cahn_implicit_2d(refine=3, dt=2.0)
    p = wl.make_problem()
    p.set_linear_params(0, tolerance_type=1, tolerance=1e-12, max_iterations=2000)
    p.set_newton_params(0, max_iterations=1, tolerance=1e-14)
    p.upload(0, wl.initial[0], age=1)
    with pytest.raises(capi.PPFError) as e:
        p.newton_solve(0)
    assert e.value.code == capi.PPF_ERR_NOCONV
    its, _, _ = p.newton_solve(0, allow_noconv=True)
    assert its == 1


def test_newton_rejects_gmg(gpu_lib):
    wl = W.allen_cahn_implicit_2d(refine=3, dt=1.0)
    p = wl.make_problem()
    p.set_linear_params(0, preconditioner=2, mg_depth=2)
    with pytest.raises(capi.PPFError) as e:
        p.newton_solve(0)
    assert e.value.code == capi.PPF_ERR_UNSUPPORTED
