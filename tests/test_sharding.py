"""The sharded explicit loop (phasefield_gb300/sharding.py) on CPU: slab partitions and halo
plans are checked exactly; the loop itself runs the oracle on every rank's slab (gloo ranks for
world size 2) and must reproduce a single oracle run of the whole mesh (1e-12 relative L2: the
same arithmetic, with node sums in a different order)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from phasefield_gb300 import sharding as S
from phasefield_gb300 import workloads as W


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


class OracleLocal:
    """The oracle on one rank's slab (the local engine of these CPU tests)."""

    device = "cpu"

    def __init__(self, oracle):
        import torch
        self.o = oracle
        self.torch = torch

    def vector(self, f: int):
        return self.torch.from_numpy(self.o.get(f, 0).copy())

    def commit(self, f: int, v):
        self.o.set(f, v.numpy(), 0)

    def increment_block(self, b: int, is_output: bool):
        rc = self.o.increment_block(b, is_output)
        if rc:
            raise RuntimeError(f"oracle block {b}: status {rc}")

    def end_increment(self) -> bool:
        return self.o.end_increment() == 2

    def get(self, f: int, age: int) -> np.ndarray:
        return self.o.get(f, age)

    def zeros(self, n: int):
        return self.torch.zeros(n, dtype=self.torch.float64)

    def apply(self, b: int, which: int, src, scale: int):
        return self.torch.from_numpy(self.o.apply(b, which, None if src is None else src.numpy(), scale))

    def set_current(self, f: int, v):
        self.o.set(f, v.numpy().copy(), 0)

    def lhs_diagonal(self, b: int, tolerance_type: int):
        self.o.set_linear_params(b, tolerance_type=tolerance_type)
        return self.torch.from_numpy(self.o.diagonal(b))

    def constrained(self, f: int) -> np.ndarray:
        kind, _, _ = self.o.constraints(f)
        perm = self.o.dealii_to_lattice(self.o.wl.fields[f].field_type)
        out = np.zeros(perm.size, dtype=bool)
        out[perm] = np.asarray(kind) != 0
        return out


def _ch(periodic=True):
    wl = W.cahn_hilliard_3d(refine=3, degree=2, dim=2, size=8.0, dt=2e-5, periodic=periodic)
    if periodic:  # a periodic initial condition along the split axis (images = masters)
        P = wl.mesh.nodes[0]
        c0 = wl.initial[0].copy()
        c0[-P:] = c0[:P]
        wl.initial = {0: c0}
    return wl


def _ac():
    return W.allen_cahn_2d(refine=4, degree=1, dt=0.01)


@pytest.mark.parametrize("size", [1, 2, 3])
@pytest.mark.parametrize("periodic", [0, 1])
@pytest.mark.parametrize("degree", [1, 2])
def test_partition_owns_every_plane_once(size, periodic, degree):
    mesh = W.RectangularMesh(dim=2, degree=degree, size=(4.0, 8.0), subdivisions=(1, 1, 1), global_refinement=3,
                             periodic=(0, periodic, 0))
    slabs = [S.partition(mesh, r, size) for r in range(size)]
    v = np.random.default_rng(0).uniform(size=int(np.prod(mesh.nodes)))
    if periodic:  # images carry their master's values
        P = mesh.nodes[0]
        v[-P:] = v[:P]
    parts = []
    for s in slabs:
        loc = S.local_from_global(s, v)
        lo, hi = s.owned_planes()
        parts.append(loc[lo * s.plane_size:hi * s.plane_size])
        # what a rank sends is what its neighbour expects in its ghost planes
        if s.left is not None:
            nb = slabs[s.left]
            a, b = s.send_left_planes()
            c, d = nb.recv_right_planes()
            assert b - a == d - c
            assert [s.global_plane(x) for x in range(a, b)] == [nb.global_plane(x) for x in range(c, d)]
        if s.right is not None:
            nb = slabs[s.right]
            a, b = s.send_right_planes()
            c, d = nb.recv_left_planes()
            assert b - a == d - c
            assert [s.global_plane(x) for x in range(a, b)] == [nb.global_plane(x) for x in range(c, d)]
    assert np.array_equal(S.assemble(slabs, parts, mesh), v)


def _run_sharded(wl, rank, size, n, every, dist_=None):
    from oracle import pyoracle as po
    slab = S.partition(wl.mesh, rank, size)
    o = po.Oracle(S.local_workload(wl, slab))
    for f, v in S.local_workload(wl, slab).initial.items():
        o.set(f, v, 0)
    run = S.ShardedExplicit(slab, OracleLocal(o), wl.fields, wl.blocks, dist_)
    run.run(n, every)
    return slab, run


@pytest.mark.parametrize("periodic", [True, False])
def test_single_rank_slab_matches_global(periodic):
    from oracle import pyoracle as po
    wl = _ch(periodic)
    n = 12
    slab, run = _run_sharded(wl, 0, 1, n, 0)
    o = po.Oracle(wl)
    assert o.run(n) == 0
    for f in (0, 1):
        got = S.assemble([slab], [run.owned(f, 1)], wl.mesh)
        assert rel_l2(got, o.get(f, 1)) < 1e-12


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, which, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        wl = _ch(True) if which == "ch" else _ac()
        n, every = (10, 0) if which == "ch" else (12, 6)
        slab, run = _run_sharded(wl, rank, world, n, every, dist)
        fields = [(0, 1), (1, 1)] if which == "ch" else [(0, 1), (1, 0), (2, 0)]
        results[rank] = [run.owned(f, a) for f, a in fields]
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("which", ["ch", "ac"])
def test_two_gloo_ranks_match_global(which):
    from oracle import pyoracle as po
    world = 2
    with mp.get_context("spawn").Manager() as m:
        results = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), which, results), nprocs=world, join=True)
        res = dict(results)
    wl = _ch(True) if which == "ch" else _ac()
    slabs = [S.partition(wl.mesh, r, world) for r in range(world)]
    o = po.Oracle(wl)
    if which == "ch":
        assert o.run(10) == 0
        refs = [o.get(0, 1), o.get(1, 1)]
    else:
        assert o.run(12, 6) == 0
        refs = [o.get(0, 1), o.get(1, 0), o.get(2, 0)]
    for i, ref in enumerate(refs):
        got = S.assemble(slabs, [res[r][i] for r in range(world)], wl.mesh)
        assert rel_l2(got, ref) < 1e-12, i


# ---------------------------------------------------------------------------------------------
# the sharded CG of a Linear block
# ---------------------------------------------------------------------------------------------
def _elasticity():
    # 4^3 Q2 cells of [0,16]^3, five inclusions, u = 0 on x = 0; two ranks own two z-layers each
    return W.eshelby_3d(refine=2, degree=2, size=16.0, n_incl=5)


LINEAR_CASES = {0: 1e-10, 1: 1e-9}  # tolerance type -> tolerance (AbsoluteResidual scaled below)


def _linear_tolerance(wl, tolerance_type):
    from oracle import pyoracle as po
    if tolerance_type == 0:  # absolute: relative to the right-hand side's norm
        return LINEAR_CASES[0] * float(np.linalg.norm(po.Oracle(wl).apply(0, 0, None, scale=0)))
    return LINEAR_CASES[tolerance_type]


CHEBYSHEV = dict(smoother_degree=4, smoothing_range=15.0, eig_cg_iterations=10)


def _run_linear(wl, rank, size, tolerance_type, dist_=None, preconditioner=0):
    from oracle import pyoracle as po
    slab = S.partition(wl.mesh, rank, size)
    o = po.Oracle(S.local_workload(wl, slab))
    run = S.ShardedLinear(slab, OracleLocal(o), wl.fields, wl.blocks, wl.mesh, dist_)
    its, res = run.solve(0, tolerance_type=tolerance_type, tolerance=_linear_tolerance(wl, tolerance_type),
                         max_iterations=2000, preconditioner=preconditioner, **CHEBYSHEV)
    return slab, its, res, run.owned(0)


def _global_linear(wl, tolerance_type, preconditioner=0):
    from oracle import pyoracle as po
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=tolerance_type, tolerance=_linear_tolerance(wl, tolerance_type),
                        max_iterations=2000, preconditioner=preconditioner, mg_depth=1, **CHEBYSHEV)
    rc, its, res = o.linear_solve(0)
    assert rc == 0
    return its, o.get(0)


def test_local_workload_drops_dirichlet_on_interior_faces():
    wl = _elasticity()
    wl.fields[0].dirichlet[(2, 5)] = 0.0  # u_z = 0 on z = 16 (the split axis' upper face)
    lows = [S.local_workload(wl, S.partition(wl.mesh, r, 2)).fields[0].dirichlet for r in range(2)]
    assert (2, 5) not in lows[0] and (2, 5) in lows[1]  # only the top slab has the global face
    assert all((c, 0) in d for d in lows for c in range(3))  # x = 0 is in every slab
    assert (2, 5) in wl.fields[0].dirichlet  # the global workload is unchanged


@pytest.mark.parametrize("tolerance_type,preconditioner", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_single_rank_sharded_cg_matches_global(tolerance_type, preconditioner):
    wl = _elasticity()
    slab, its, res, part = _run_linear(wl, 0, 1, tolerance_type, preconditioner=preconditioner)
    oits, ref = _global_linear(wl, tolerance_type, preconditioner)
    assert abs(its - oits) <= 2, (its, oits)
    assert rel_l2(S.assemble([slab], [part], wl.mesh, ncomp=3), ref) < 1e-8


def _linear_worker(rank, world, port, tolerance_type, preconditioner, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=120))
    try:
        _, its, res, part = _run_linear(_elasticity(), rank, world, tolerance_type, dist, preconditioner)
        results[rank] = (its, res, part)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("tolerance_type,preconditioner", [(0, 0), (1, 1)])
def test_two_gloo_ranks_sharded_cg_matches_global(tolerance_type, preconditioner):
    world = 2
    with mp.get_context("spawn").Manager() as m:
        results = m.dict()
        mp.spawn(_linear_worker, args=(world, _free_port(), tolerance_type, preconditioner, results), nprocs=world,
                 join=True)
        res = dict(results)
    wl = _elasticity()
    slabs = [S.partition(wl.mesh, r, world) for r in range(world)]
    oits, ref = _global_linear(wl, tolerance_type, preconditioner)
    assert res[0][0] == res[1][0]  # every rank ran the same iterations
    assert abs(res[0][0] - oits) <= 2, (res[0][0], oits)
    got = S.assemble(slabs, [res[r][2] for r in range(world)], wl.mesh, ncomp=3)
    assert rel_l2(got, ref) < 1e-8
