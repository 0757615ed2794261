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
