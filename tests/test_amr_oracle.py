"""Adaptive meshes in the oracle: the properties its restatement of RefinementManager
(src/core/refinement_manager.cc), deal.II's hanging-node constraints and SolutionTransfer must
have, checked on the CPU. The GPU engine is compared with this oracle in test_gpu_amr.py."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import workloads as W


def _run0(wl, adaptivity=None):
    o = po.Oracle(wl, adaptivity=adaptivity or wl.adaptivity)
    assert o.run(0, 0) == 0
    return o


def _cases():
    return [
        ("ac2_q2", lambda: W.allen_cahn_amr_2d(refine=3, degree=2, min_level=2, max_level=5)),
        ("ac2_q1", lambda: W.allen_cahn_amr_2d(refine=3, degree=1, min_level=2, max_level=6)),
        ("ch2_q2_periodic", lambda: W.cahn_hilliard_amr(2)),
        ("ch3_q1_periodic", lambda: W.cahn_hilliard_amr(3, refine=2, degree=1, max_level=4, size=16.0,
                                                          gradient_bound=0.1)),
    ]


def _spans(o, wl):
    """per cell: lower corner and width in node units at the finest level"""
    cells = o.cells()
    M = wl.adaptivity["max_level"]
    k = wl.mesh.degree
    w = (k << (M - cells[:, 0])).astype(np.int64)
    lo = cells[:, 1:1 + wl.mesh.dim].astype(np.int64) * w[:, None]
    return cells, lo, w


def _extent(wl):
    M = wl.adaptivity["max_level"]
    return [(wl.mesh.subdivisions[d] * wl.mesh.degree) << M for d in range(wl.mesh.dim)]


@pytest.mark.parametrize("name,make", _cases(), ids=[c[0] for c in _cases()])
def test_cells_tile_the_domain_and_are_balanced(name, make):
    wl = make()
    o = _run0(wl)
    cells, lo, w = _spans(o, wl)
    dim = wl.mesh.dim
    E = _extent(wl)
    assert len(np.unique(cells[:, 0])) > 1, "the mesh should have been graded"
    # cells tile the domain: volumes add up and no two cells overlap
    assert int((w.astype(np.float64) ** dim).sum()) == int(np.prod(E))
    # 2:1 balance between every pair of cells that share at least a vertex
    n = len(cells)
    touch = np.ones((n, n), bool)
    for d in range(dim):
        a0, a1 = lo[:, d][:, None], (lo[:, d] + w)[:, None]
        hit = np.zeros((n, n), bool)
        shifts = [-E[d], 0, E[d]] if wl.mesh.periodic[d] else [0]
        for sh in shifts:
            b0, b1 = lo[:, d][None, :] + sh, (lo[:, d] + w)[None, :] + sh
            hit |= (a0 <= b1) & (b0 <= a1)
        touch &= hit
    np.fill_diagonal(touch, False)
    lev = cells[:, 0]
    assert np.abs(lev[:, None] - lev[None, :])[touch].max() <= 1
    # tree order: the ancestors' child digits (x fastest) increase depth-first
    M = wl.adaptivity["max_level"]
    keys = []
    for l, x, y, z in cells:
        coarse = [int(v) >> int(l) for v in (x, y, z)[:dim]]
        cidx = coarse[0] + wl.mesh.subdivisions[0] * (coarse[1] + (wl.mesh.subdivisions[1] * coarse[2] if dim == 3 else 0))
        path = 0
        for t in range(1, M + 1):
            digit = 0
            if t <= l:
                for d, v in enumerate((x, y, z)[:dim]):
                    digit |= ((int(v) >> (int(l) - t)) & 1) << d
            path = (path << dim) | digit
        keys.append((cidx, path))
    assert keys == sorted(keys)


@pytest.mark.parametrize("name,make", _cases(), ids=[c[0] for c in _cases()])
def test_hanging_lines_reproduce_the_element_polynomials(name, make):
    wl = make()
    o = _run0(wl)
    k = wl.mesh.degree
    x = o.node_points()
    cnt, mas, wts = o.hanging()
    assert (cnt > 0).sum() > 0
    off = np.concatenate([[0], np.cumsum(cnt)])
    # lines whose masters lie across a periodic seam see a polynomial jump there: skip them
    hang = np.array([p for p in np.nonzero(cnt)[0]
                     if (np.abs(x[mas[off[p]:off[p + 1]]] - x[p]).max(0)[:wl.mesh.dim]
                         < 0.5 * np.asarray(wl.mesh.size[:wl.mesh.dim])).all()])
    assert len(hang) > 0
    # every tensor-product monomial of degree <= k per variable is interpolated exactly
    for powers in itertools.product(range(k + 1), repeat=wl.mesh.dim):
        f = np.ones(len(x))
        for d, p in enumerate(powers):
            f = f * (1.0 + x[:, d] / wl.mesh.size[d]) ** p
        vals = np.array([(wts[off[p]:off[p + 1]] * f[mas[off[p]:off[p + 1]]]).sum() for p in hang])
        assert np.abs(vals - f[hang]).max() <= 1e-13 * np.abs(f).max()
    # masters are never hanging themselves (closed lines)
    assert (cnt[mas] == 0).all()


def test_numbering_is_first_touch_over_tree_order():
    wl = W.allen_cahn_amr_2d(refine=3, degree=2, min_level=2, max_level=5)
    o = _run0(wl)
    cd = o.cell_dofs(0)
    first = np.full(o.n_nodes(), -1)
    order = []
    for i, d in enumerate(cd):
        if first[d] < 0:
            first[d] = i
            order.append(d)
    assert order == list(range(o.n_nodes()))


@pytest.mark.parametrize("value", [0.0, 1.0])
def test_allen_cahn_constants_stay_fixed_across_levels(value):
    wl = W.allen_cahn_amr_2d(refine=3, degree=2, min_level=2, max_level=5)
    o = _run0(wl)
    n = o.n_nodes()
    o.set_native(0, np.full(n, value), 0)
    o.set_native(0, np.full(n, value), 1)
    o.solve_block(0)
    assert np.abs(o.get_native(0) - value).max() < 1e-14


@pytest.mark.parametrize("dim,degree", [(2, 1), (2, 2), (3, 1)])
def test_cahn_hilliard_conserves_mass_on_a_graded_periodic_mesh(dim, degree):
    wl = W.cahn_hilliard_amr(dim, refine=2 if dim == 3 else 3, degree=degree, max_level=4 if dim == 3 else 5,
                             size=16.0 if dim == 3 else 32.0, gradient_bound=0.25 if (dim, degree) == (2, 2) else 0.1)
    ad = dict(wl.adaptivity, period=0)
    o = po.Oracle(wl, adaptivity=ad)
    assert o.run(0, 0) == 0
    assert len(np.unique(o.cells()[:, 0])) > 1
    invm = o.invm_native(0)
    jxw = np.where(invm > 0, 1.0 / np.where(invm > 0, invm, 1.0), 0.0)
    # the condensed lumped mass integrates the finite-element function exactly for a constant
    assert abs(jxw.sum() - np.prod(wl.mesh.size[:dim])) < 1e-10 * np.prod(wl.mesh.size[:dim])
    m0 = (jxw * o.get_native(0, 1)).sum()
    assert o.run(20, 0) == 0
    m1 = (jxw * o.get_native(0, 1)).sum()
    assert abs(m1 - m0) < 1e-12 * abs(m0)


def test_transfer_keeps_fields_the_mesh_can_represent():
    wl = W.allen_cahn_amr_2d(refine=3, degree=2, min_level=2, max_level=5)
    o = _run0(wl)
    L = wl.mesh.size[0]
    poly = lambda x: 1.0 + 0.5 * (x[:, 0] / L) - 0.25 * (x[:, 1] / L) ** 2 + 0.75 * (x[:, 0] / L) * (x[:, 1] / L)
    # move the interfaces (field 0) so that the next pass refines and coarsens elsewhere, and
    # give field 1 a quadratic, which every mesh of the hierarchy represents exactly
    for _ in range(2):
        x = o.node_points()
        o.set_native(0, 0.5 + 0.49 * np.sin(2 * np.pi * x[:, 0] / L + 1.3) * np.cos(2 * np.pi * x[:, 1] / L))
        o.set_native(1, poly(x))
        before = o.cells()
        o.adapt()
        after = o.cells()
        assert before.shape != after.shape or (before != after).any()
        assert np.abs(o.get_native(1) - poly(o.node_points())).max() < 1e-13


def test_adaptive_mesh_at_one_level_matches_the_uniform_oracle():
    wl = W.cahn_hilliard_amr(2, refine=3, degree=2)
    ad = dict(min_level=3, max_level=3, period=1, criteria=[(0, 2, 0.0, 0.0, 0.25)])
    a = po.Oracle(wl, adaptivity=ad)
    u = po.Oracle(wl)
    for o in (a, u):
        assert o.run(6, 0) == 0
    for f in (0, 1):
        ref = a.lattice_to_native(f, u.get(f, 1))
        assert np.abs(a.get_native(f, 1) - ref).max() < 1e-13
