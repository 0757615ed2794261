"""GPU tests of the batched ensemble: every instance of one-launch-per-step ensemble runs must
match the same simulation run alone through a handle (one FP64 step is the same arithmetic,
so 1e-12 relative L2 after a few steps), with and without the captured graph, and after the
autotuner has picked a tile shape."""
import numpy as np
import pytest

from phasefield_gb300 import ensemble as E
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-11


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def single(mesh, m_well, kappa, ic, dt, steps):
    wl = W.allen_cahn_2d(degree=mesh.degree, refine=mesh.global_refinement, m_well=m_well, kappa=kappa, dt=dt,
                         subdivisions=mesh.subdivisions[:2])
    wl.initial = {0: ic}
    p = wl.make_problem()
    p.solve(steps)
    out = p.download(0, age=1)
    p.close()
    return out


@pytest.mark.parametrize("use_graph", [False, True])
def test_ensemble_matches_single_simulations(gpu_lib, use_graph):
    meshes, mw, ka, ics = E.allen_cahn_ensemble(n_instances=6, min_cells=8, max_cells=40, seed=7)
    dt, steps = 0.01, 7
    ens = E.Ensemble(meshes, mw, ka, dt)
    for i, ic in enumerate(ics):
        ens.upload(i, ic)
    ens.run(steps, use_graph=use_graph)
    for i in range(len(meshes)):
        ref = single(meshes[i], mw[i], ka[i], ics[i], dt, steps)
        assert rel_l2(ens.download(i), ref) < TOL, i


def test_autotune_keeps_state_and_results(gpu_lib):
    meshes, mw, ka, ics = E.allen_cahn_ensemble(n_instances=8, min_cells=8, max_cells=48, seed=11)
    dt, steps = 0.01, 5
    ens = E.Ensemble(meshes, mw, ka, dt)
    for i, ic in enumerate(ics):
        ens.upload(i, ic)
    ms, shape, grid = ens.autotune(steps=2)
    assert ms > 0 and shape in (0, 1, 2) and grid in (1, 2, 4, 8)
    for i, ic in enumerate(ics):  # state restored by the autotuner
        assert rel_l2(ens.download(i), ic) < 1e-14
    ens.run(steps, use_graph=True)
    for i in range(len(meshes)):
        ref = single(meshes[i], mw[i], ka[i], ics[i], dt, steps)
        assert rel_l2(ens.download(i), ref) < TOL, i
