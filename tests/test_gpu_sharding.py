"""The sharded explicit loop on the GPU engine (one rank: the periodic split axis exchanges with
itself through device tensors on torch's stream) against the plain engine loop. Bar: 1e-12
relative L2 (same kernels; the slab adds ghost cells whose sums reach owned nodes in a
different order)."""
import numpy as np
import pytest

from phasefield_gb300 import sharding as S
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _periodic_ic(wl):
    P = int(np.prod(wl.mesh.nodes[:-1]))
    v = wl.initial[0].copy()
    v[-P:] = v[:P]  # periodic along the split axis
    wl.initial = {**wl.initial, 0: v}
    return wl


@pytest.mark.parametrize("case", ["ch3d", "ac2d"])
def test_sharded_engine_one_rank_matches_plain(gpu_lib, case):
    import torch
    if case == "ch3d":
        wl = _periodic_ic(W.cahn_hilliard_3d(refine=2, degree=2, size=4.0, dt=1e-4))
        n, every, fields = 12, 0, [(0, 1), (1, 1)]
    else:
        wl = W.allen_cahn_2d(refine=4, degree=1, dt=0.01)
        n, every, fields = 12, 6, [(0, 1), (1, 0), (2, 0)]
    ref = wl.make_problem()
    ref.solve(n, output_every=every)
    slab = S.partition(wl.mesh, 0, 1)
    lw = S.local_workload(wl, slab)
    p = lw.make_problem()
    run = S.ShardedExplicit(slab, S.EngineLocal(p), wl.fields, wl.blocks)
    run.run(n, every)
    torch.cuda.synchronize()
    for f, age in fields:
        got = S.assemble([slab], [run.owned(f, age)], wl.mesh)
        assert rel_l2(got, ref.download(f, age=age)) < 1e-12, (f, age)


@pytest.mark.parametrize("tolerance_type,preconditioner", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_sharded_cg_engine_one_rank_matches_plain_cg(gpu_lib, tolerance_type, preconditioner):
    """The sharded CG of the elasticity block (device vectors, halo exchange with itself, owned
    inner products), without a preconditioner and with the Chebyshev one, against the engine's
    own CG with the same preconditioner: same iteration count within 2, solutions within 1e-8."""
    import torch
    cheb = dict(smoother_degree=4, smoothing_range=15.0, eig_cg_iterations=10)
    wl = W.eshelby_3d(refine=2, degree=2, size=16.0, n_incl=5)
    ref = wl.make_problem()
    b = ref.apply(0, 0, None, scale=0)
    tol = 1e-10 * float(np.linalg.norm(b)) if tolerance_type == 0 else 1e-9
    ref.set_linear_params(0, tolerance_type=tolerance_type, tolerance=tol, max_iterations=2000,
                          preconditioner=preconditioner, mg_depth=1, **cheb)
    its_ref, _ = ref.linear_solve(0)
    slab = S.partition(wl.mesh, 0, 1)
    p = S.local_workload(wl, slab).make_problem()
    run = S.ShardedLinear(slab, S.EngineLocal(p), wl.fields, wl.blocks, wl.mesh)
    its, res = run.solve(0, tolerance_type=tolerance_type, tolerance=tol, max_iterations=2000,
                         preconditioner=preconditioner, **cheb)
    torch.cuda.synchronize()
    assert abs(its - its_ref) <= 2, (its, its_ref)
    got = S.assemble([slab], [run.owned(0)], wl.mesh, ncomp=3)
    assert rel_l2(got, ref.download(0)) < 1e-8
