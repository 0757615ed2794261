"""Generates the golden fixtures of this directory from the oracle (run from the repository root):

  python tests/golden/make_golden.py

The reference's own tests hold no vectors for the operator-evaluation path, so these are
seeded oracle dumps at small instances of the benchmark configurations: deal.II DoF maps,
constraint maps, the lumped inverse mass, one operator apply, fields after N explicit steps,
the operator diagonal and a preconditioned CG solution with its iteration count; and an
adaptive mesh's cells, DoF table, hanging-node lines and fields after remeshing increments. The CPU tests
check that the oracle still reproduces them; the GPU tests check the CUDA path against them.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import pyoracle as po  # noqa: E402
from phasefield_gb300 import workloads as W  # noqa: E402


def cmap_lattice(o, f):
    """Constraint map in lattice order: master index (itself if free) or -1 for Dirichlet."""
    kind, master, _ = o.constraints(f)
    perm = o.dealii_to_lattice(o.wl.fields[f].field_type)
    out = np.empty(perm.size, dtype=np.int64)
    for i in range(perm.size):
        out[perm[i]] = perm[i] if not kind[i] else (perm[master[i]] if master[i] >= 0 else -1)
    return out


# the workloads of the fixtures (also used by the tests that read them)
def wl_allen_cahn():
    return W.allen_cahn_2d(refine=4, degree=2, dt=0.01, seed=11)


def wl_cahn_hilliard():
    return W.cahn_hilliard_3d(refine=1, degree=2, size=2.0, dt=2e-4, seed=12)


def wl_coupled():
    return W.coupled_acch_2d(refine=4, degree=2, size=64.0, dt=1e-3, seed=13)


def wl_elasticity():
    return W.eshelby_3d(refine=1, degree=2, size=8.0, n_incl=3, seed=14)


def wl_allen_cahn_amr():
    return W.allen_cahn_amr_2d(refine=3, degree=2, min_level=2, max_level=5, period=5, seed=16, n_grains=6)


ELASTICITY_SOLVER = dict(tolerance_type=0, tolerance=1e-11, max_iterations=500, preconditioner=2, mg_depth=2,
                         smoother_degree=4)


def allen_cahn():
    wl = wl_allen_cahn()
    o = po.Oracle(wl)
    d = dict(dof_map=o.dealii_to_lattice(0), invm=o.invm(0), n0=wl.initial[0])
    o.set(0, wl.initial[0], age=1)
    d["rhs_apply"] = o.apply(0, 0, None, scale=1)
    o2 = po.Oracle(wl)
    assert o2.run(25, 25) == 0
    d.update(n_25=o2.get(0, 1), mg_n_25=o2.get(1, 0), f_tot_25=o2.get(2, 0))
    return d


def cahn_hilliard():
    wl = wl_cahn_hilliard()
    o = po.Oracle(wl)
    d = dict(cmap=cmap_lattice(o, 0), invm=o.invm(0), c0=wl.initial[0])
    assert o.run(10) == 0
    d.update(c_10=o.get(0, 1), mu_10=o.get(1, 1))
    return d


def coupled():
    wl = wl_coupled()
    o = po.Oracle(wl)
    assert o.run(12, 6) == 0
    return dict(c0=wl.initial[0], n0=wl.initial[1], c_12=o.get(0, 1), n_12=o.get(1, 1), f_tot_12=o.get(2, 0),
                mag_grad_c_12=o.get(3, 0))


def elasticity():
    wl = wl_elasticity()
    o = po.Oracle(wl)
    rng = np.random.default_rng(15)
    src = rng.uniform(-1.0, 1.0, o.n_dofs(1))
    d = dict(vector_dof_map=o.dealii_to_lattice(1), cmap=cmap_lattice(o, 0), src=src,
             lhs_apply=o.apply(0, 1, src, scale=0), rhs_apply=o.apply(0, 0, None, scale=0))
    o.set_linear_params(0, **ELASTICITY_SOLVER)
    d["diagonal"] = o.diagonal(0)
    rc, its, res = o.linear_solve(0)
    assert rc == 0
    d.update(u=o.get(0, 0), iterations=np.int64(its), residual=np.float64(res))
    return d


def allen_cahn_amr():
    """Adaptive mesh: the active cells, DoF table, hanging-node lines, lumped mass and fields
    after 12 increments with the initial refinement and remeshing every 5 increments."""
    wl = wl_allen_cahn_amr()
    o = po.Oracle(wl, adaptivity=wl.adaptivity)
    assert o.run(12, 12) == 0
    cnt, mas, w = o.hanging()
    return dict(n0=wl.initial[0], cells=o.cells().astype(np.int64), cell_dofs=o.cell_dofs(0),
                hang_count=cnt.astype(np.int64), hang_master=mas, hang_weight=w, invm=o.invm_native(0),
                n_12=o.get_native(0, 1), mg_n_12=o.get_native(1, 0), f_tot_12=o.get_native(2, 0))


FIXTURES = {"allen_cahn_2d_q2": allen_cahn, "allen_cahn_amr_2d_q2": allen_cahn_amr, "cahn_hilliard_3d_q2": cahn_hilliard, "coupled_acch_2d_q2": coupled,
            "elasticity_3d_q2": elasticity}


def main():
    for name, fn in FIXTURES.items():
        d = fn()
        np.savez_compressed(HERE / f"{name}.npz", **d)
        print(name, {k: np.shape(v) for k, v in d.items()})


if __name__ == "__main__":
    main()
