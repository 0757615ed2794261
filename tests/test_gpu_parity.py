"""GPU parity tests: the CUDA path through the C ABI against the oracle on the same seeded inputs.

Bars (stated per test): DoF maps, connectivity and constraint maps bit-exact; one FP64
operator apply within 1e-12 relative L2; fields after N explicit steps within 1e-9 relative L2.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W
from phasefield_gb300.problem import (Explicit, FieldAttributes, Linear, Primary, RectangularMesh, Scalar,
                                      SolveBlock, Vector, make_dependency_set)

pytestmark = pytest.mark.gpu

APPLY_TOL = 1e-12
STEPS_TOL = 1e-9


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def eshelby_small(dim=3, degree=2, refine=2, n_incl=5):
    wl = W.eshelby_3d(refine=refine, degree=degree, size=16.0, n_incl=n_incl, dim=dim)
    return wl


# ---------------------------------------------------------------------------------------------
# maps
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("dim,degree,refine,sub", [(2, 1, 2, (1, 1, 1)), (2, 2, 1, (2, 3, 1)), (2, 3, 1, (1, 1, 1)),
                                                    (2, 4, 1, (1, 2, 1)), (3, 1, 2, (1, 1, 1)), (3, 2, 1, (2, 1, 1)),
                                                    (3, 3, 1, (1, 2, 1)), (3, 4, 1, (1, 1, 2))])
def test_dof_map_bit_exact(gpu_lib, dim, degree, refine, sub):
    wl = W.cahn_hilliard_3d(refine=refine, degree=degree, dim=dim, size=2.0, subdivisions=sub, periodic=False)
    wl.mesh.size = tuple(float(s) for s in sub[:dim]) + (1.0,) * (3 - dim)
    p = wl.make_problem()
    o = po.Oracle(wl)
    assert np.array_equal(p.dof_map(0), o.dealii_to_lattice(0))


@pytest.mark.parametrize("dim,degree", [(2, 2), (3, 1), (3, 2)])
def test_vector_dof_map_bit_exact(gpu_lib, dim, degree):
    wl = eshelby_small(dim=dim, degree=degree, refine=1)
    p = wl.make_problem()
    o = po.Oracle(wl)
    assert np.array_equal(p.dof_map(1), o.dealii_to_lattice(1))


def _oracle_cmap_lattice(o, f):
    """Oracle constraints expressed like the product's map: master lattice index or -1-row."""
    kind, master, inhom = o.constraints(f)
    perm = o.dealii_to_lattice(o.wl.fields[f].field_type)
    out = np.empty(perm.size, dtype=np.int64)
    vals = np.full(perm.size, np.nan)
    for i in range(perm.size):
        li = perm[i]
        if not kind[i]:
            out[li] = li
        elif master[i] >= 0:
            out[li] = perm[master[i]]
        else:
            out[li] = -1
            vals[li] = inhom[i]
    return out, vals


def test_periodic_constraint_map_bit_exact(gpu_lib):
    wl = W.cahn_hilliard_3d(refine=2, degree=2, size=4.0)
    p = wl.make_problem()
    o = po.Oracle(wl)
    ref, _ = _oracle_cmap_lattice(o, 0)
    got = p.constraint_map(0).astype(np.int64)
    assert np.array_equal(got, ref)


def test_dirichlet_constraint_map_bit_exact(gpu_lib):
    wl = eshelby_small(dim=3, degree=2, refine=1)
    # u = 0 on x = 0 (boundary id 0) and u_x = 0.05 on x = 16 (boundary id 1): nonzero values
    wl.fields[0].dirichlet[(0, 1)] = 0.05
    p = wl.make_problem()
    o = po.Oracle(wl)
    ref, vals = _oracle_cmap_lattice(o, 0)
    got = p.constraint_map(0).astype(np.int64)
    assert np.array_equal(got >= 0, ref >= 0)
    assert np.array_equal(got[got >= 0], ref[got >= 0])
    # the values: distributing the constraints on a zero vector leaves exactly the Dirichlet
    # values in the constrained rows (AffineConstraints::distribute)
    p.upload(0, np.zeros(p.field_length(0)))
    p.apply_constraints(0)
    u = p.download(0)
    rows = ref < 0
    assert rows.sum() > 0 and np.any(vals[rows] != 0.0)
    assert np.array_equal(u[rows], vals[rows])
    assert np.all(u[~rows] == 0.0)


def test_invm_matches(gpu_lib):
    wl = W.cahn_hilliard_3d(refine=2, degree=2, size=4.0)
    p = wl.make_problem()
    o = po.Oracle(wl)
    assert rel_l2(p.invm(), o.invm(0)) < 1e-14


# ---------------------------------------------------------------------------------------------
# one operator apply
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("degree", [1, 2, 3, 4])
def test_allen_cahn_rhs_apply(gpu_lib, degree):
    wl = W.allen_cahn_2d(refine=4, degree=degree)
    p = wl.make_problem()
    o = po.Oracle(wl)
    n0 = wl.initial[0]
    p.upload(0, n0, age=1)
    o.set(0, n0, age=1)
    for scale in (0, 1):
        got = p.apply(0, 0, None, scale=scale)
        ref = o.apply(0, 0, None, scale=scale)
        assert rel_l2(got, ref) < APPLY_TOL


@pytest.mark.parametrize("dim,degree", [(2, 2), (3, 1), (3, 2), (3, 3), (3, 4)])
def test_cahn_hilliard_block_applies(gpu_lib, dim, degree):
    wl = W.cahn_hilliard_3d(refine=2 if dim == 3 else 4, degree=degree, dim=dim, size=8.0)
    p = wl.make_problem()
    o = po.Oracle(wl)
    rng = np.random.default_rng(3)
    N = p.n_nodes
    c, mu = wl.initial[0], rng.uniform(-1, 1, N)
    for f, v in ((0, c), (1, mu)):
        p.upload(f, v, age=1)
        o.set(f, v, age=1)
    p.upload(0, c, age=0)
    o.set(0, c, age=0)
    for b in (0, 1):
        got = p.apply(b, 0, None, scale=1)
        ref = o.apply(b, 0, None, scale=1)
        assert rel_l2(got, ref) < APPLY_TOL, b


@pytest.mark.parametrize("dim,degree", [(2, 2), (3, 1), (3, 2)])
def test_eshelby_lhs_and_rhs_apply(gpu_lib, dim, degree):
    wl = eshelby_small(dim=dim, degree=degree, refine=2 if dim == 3 else 3)
    p = wl.make_problem()
    o = po.Oracle(wl)
    rng = np.random.default_rng(11)
    u = rng.uniform(-1, 1, p.field_length(0))
    for scale in (0, 2):
        got = p.apply(0, 1, u, scale=scale)
        ref = o.apply(0, 1, u, scale=scale)
        assert rel_l2(got, ref) < APPLY_TOL
    got = p.apply(0, 0, None)
    ref = o.apply(0, 0, None)
    assert rel_l2(got, ref) < APPLY_TOL


# ---------------------------------------------------------------------------------------------
# explicit time stepping
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("degree", [1, 2, 3, 4])
def test_allen_cahn_steps(gpu_lib, degree):
    wl = W.allen_cahn_2d(refine=4, degree=degree, dt=0.01)
    p = wl.make_problem()
    o = po.Oracle(wl)
    n = 40
    p.solve(n, output_every=20)
    assert o.run(n, 20) == 0
    for f in (0, 1, 2):  # n and the postprocessed fields
        age = 1 if f == 0 else 0
        got = p.download(f, age=age) if f == 0 else p.download(f)
        ref = o.get(f, age)
        assert rel_l2(got, ref) < STEPS_TOL, f


@pytest.mark.parametrize("dim,degree", [(2, 1), (2, 2), (3, 1), (3, 2), (3, 3), (3, 4)])
def test_cahn_hilliard_steps_periodic(gpu_lib, dim, degree):
    # time steps at about a third of the explicit stability limit of each discretisation (Q3
    # and Q4 in 3-D: well inside it, the closer Gauss-Lobatto points make them stiffer)
    dt = {(2, 1): 5e-4, (2, 2): 1.5e-5, (3, 1): 2e-4, (3, 2): 1e-4, (3, 3): 2e-6, (3, 4): 5e-7}[(dim, degree)]
    wl = W.cahn_hilliard_3d(refine=2 if dim == 3 else 4, degree=degree, dim=dim, size=8.0 if dim == 2 else 4.0,
                            dt=dt)
    p = wl.make_problem()
    o = po.Oracle(wl)
    n = 30
    p.solve(n)
    assert o.run(n) == 0
    for f in (0, 1):
        assert rel_l2(p.download(f, age=1), o.get(f, 1)) < STEPS_TOL


def test_coupled_two_field_block_steps(gpu_lib):
    wl = W.coupled_acch_2d(refine=4, degree=2, size=32.0, dt=1e-3)
    p = wl.make_problem()
    o = po.Oracle(wl)
    n = 20
    p.solve(n, output_every=10)
    assert o.run(n, 10) == 0
    for f in (0, 1):
        assert rel_l2(p.download(f, age=1), o.get(f, 1)) < STEPS_TOL
    for f in (2, 3):
        assert rel_l2(p.download(f), o.get(f, 0)) < STEPS_TOL


@pytest.mark.parametrize("which", ["ch", "acch"])
def test_graph_replay_matches_plain_launches(gpu_lib, which):
    if which == "ch":
        wl = W.cahn_hilliard_3d(refine=2, degree=2, size=4.0, dt=1e-4)
    else:
        wl = W.coupled_acch_2d(refine=4, degree=2, size=32.0, dt=1e-3)
    res = []
    for use_graph in (0, 1):
        p = wl.make_problem()
        p.lib.ppf_set_use_graph(p.h, use_graph)
        p.solve(23)
        res.append([p.download(f, age=1) for f in (0, 1)])
        assert p.get_time()[0] == 24
        p.close()
    for a, b in zip(res[0], res[1]):
        assert rel_l2(b, a) < 1e-12


def test_dealii_ordering_roundtrip(gpu_lib):
    wl = W.cahn_hilliard_3d(refine=1, degree=2, size=2.0)
    p = wl.make_problem()
    o = po.Oracle(wl)
    perm = o.dealii_to_lattice(0)
    v = np.random.default_rng(5).uniform(size=p.n_nodes)
    p.upload(0, v[perm], ordering=capi.ORDER_DEALII)  # deal.II-ordered host vector
    assert np.array_equal(p.download(0), v)
    assert np.array_equal(p.download(0, ordering=capi.ORDER_DEALII), v[perm])


# ---------------------------------------------------------------------------------------------
# failure detection (host-planted faults; the GPU never faults)
# ---------------------------------------------------------------------------------------------
def test_nan_in_state_reports_ppf_err_nan(gpu_lib):
    wl = W.allen_cahn_2d(refine=3, degree=1)
    v = wl.initial[0].copy()
    v[17] = np.nan
    wl.initial = {0: v}
    p = wl.make_problem()
    with pytest.raises(capi.PPFError) as e:
        p.solve(3)
    assert e.value.code == capi.PPF_ERR_NAN


def test_undeclared_dependency_reports_error(gpu_lib):
    wl = W.allen_cahn_2d(refine=3, degree=1)
    # the callback reads old_1(n) but the block only declares the current value of n
    wl.blocks[0].dependencies_rhs = make_dependency_set(wl.fields, {"n"})
    p = wl.make_problem()
    with pytest.raises(capi.PPFError) as e:
        p.solve(2)
    assert e.value.code == capi.PPF_ERR_DEPENDENCY
