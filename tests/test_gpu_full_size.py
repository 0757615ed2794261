"""The benchmark configurations at their full size, through the C ABI, against the oracle.

* Allen-Cahn 2-D: [0,100]^2, 128^2 Q1 cells, seeded grains, dt 0.01, 1000 increments with the
  post-processed fields on the last one: fields within 1e-9 relative L2.
* Cahn-Hilliard 3-D: [0,64]^3, 64^3 Q2 cells (129^3 nodes per field), periodic, dt 1e-4: one
  FP64 apply of each block within 1e-12 relative L2 on the seeded state, then c and mu after 200
  increments (the benchmarked workload end to end) within 1e-9.
* Elasticity 3-D: [0,64]^3, Q2 vector, 40 seeded inclusions, u = 0 on x = 0, GMG-CG with
  Chebyshev degree 4 to ||b - A x|| <= 1e-10 ||b|| (the benchmark's criterion), plain FP64 and
  FP32 smoothing/transfers inside FP64 CG: solutions within 1e-8 of the oracle's, iteration
  counts within 10 % (or 2). At 32^3 cells with mg depth 6 and at the full 64^3 cells with mg
  depth 7 (6.44 M unknowns).
* Ensemble: instances of a batched run against the oracle run of each instance's own problem.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import ensemble as E
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu

APPLY_TOL = 1e-12
STEPS_TOL = 1e-9
SOLVE_TOL = 1e-8


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_allen_cahn_128_q1_1000_steps(gpu_lib):
    wl = W.allen_cahn_2d()  # 128^2 Q1, 1000 steps of dt 0.01
    assert wl.mesh.cells[:2] == [128, 128] and wl.n_steps == 1000
    p = wl.make_problem()
    p.solve(wl.n_steps, output_every=wl.n_steps)
    o = po.Oracle(wl)
    assert o.run(wl.n_steps, wl.n_steps) == 0
    assert rel_l2(p.download(0, age=1), o.get(0, 1)) < STEPS_TOL
    for f in (1, 2):  # mg_n and f_tot of the last increment
        assert rel_l2(p.download(f), o.get(f, 0)) < STEPS_TOL, f


def test_cahn_hilliard_64_q2_apply_and_200_steps(gpu_lib):
    wl = W.cahn_hilliard_3d()  # [0,64]^3, 64^3 Q2 cells, periodic, dt 1e-4, 200 steps
    assert wl.mesh.cells == [64, 64, 64] and wl.n_steps == 200
    p = wl.make_problem()
    o = po.Oracle(wl)
    assert p.n_nodes == 129 ** 3
    c0 = wl.initial[0]
    mu0 = np.random.default_rng(17).uniform(-0.1, 0.1, p.n_nodes)
    for f, v in ((0, c0), (1, mu0)):
        p.upload(f, v, age=1)
        o.set(f, v, age=1)
    p.upload(0, c0, age=0)
    o.set(0, c0, age=0)
    for b in (0, 1):  # c block (old c, grad old mu) and mu block (c, grad c), invM applied
        assert rel_l2(p.apply(b, 0, None, scale=1), o.apply(b, 0, None, scale=1)) < APPLY_TOL, b
    p.close()

    p = wl.make_problem()
    o = po.Oracle(wl)
    p.solve(wl.n_steps)
    assert o.run(wl.n_steps) == 0
    for f in (0, 1):
        assert rel_l2(p.download(f, age=1), o.get(f, 1)) < STEPS_TOL, f


def _elasticity_vs_oracle(refine, depth):
    wl = W.eshelby_3d(refine=refine, degree=2, size=64.0, n_incl=40)
    o = po.Oracle(wl)
    bnorm = float(np.linalg.norm(o.apply(0, 0, None, scale=0)))
    prm = dict(tolerance_type=0, tolerance=1e-10 * bnorm, max_iterations=500, preconditioner=2, mg_depth=depth,
               smoother_degree=4)
    o.set_linear_params(0, **prm)
    rc, oits, _ = o.linear_solve(0)
    assert rc == 0
    ref = o.get(0)
    for mixed in (0, 1):
        p = wl.make_problem()
        p.set_linear_params(0, mixed_precision=mixed, **prm)
        its, res = p.linear_solve(0)
        assert res <= 1e-10 * bnorm, mixed
        assert abs(its - oits) <= max(2, 0.1 * oits), (mixed, its, oits)
        assert rel_l2(p.download(0), ref) < SOLVE_TOL, mixed
        p.close()


def test_elasticity_32_q2_gmg_depth6_fp64_and_mixed(gpu_lib):
    _elasticity_vs_oracle(5, 6)


def test_elasticity_64_q2_gmg_depth7_fp64_and_mixed(gpu_lib):
    _elasticity_vs_oracle(6, 7)


def test_ensemble_instances_match_oracle(gpu_lib):
    meshes, mw, ka, ics = E.allen_cahn_ensemble(n_instances=6, min_cells=16, max_cells=96, seed=5)
    dt, steps = 0.01, 25
    ens = E.Ensemble(meshes, mw, ka, dt)
    for i, ic in enumerate(ics):
        ens.upload(i, ic)
    ens.run(steps, use_graph=True)
    assert {m.degree for m in meshes} == {1, 2}
    for i, m in enumerate(meshes):
        wl = W.allen_cahn_2d(degree=m.degree, refine=m.global_refinement, m_well=mw[i], kappa=ka[i], dt=dt,
                             subdivisions=m.subdivisions[:2], size=m.size[0])
        assert wl.mesh.cells[:2] == m.cells[:2]
        wl.initial = {0: ics[i]}
        o = po.Oracle(wl)
        assert o.run(steps) == 0
        assert rel_l2(ens.download(i), o.get(0, 1)) < STEPS_TOL, i
