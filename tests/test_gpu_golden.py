"""The CUDA path, through the C ABI, against the committed golden fixtures (tests/golden).

Bars as in the parity tests: index and constraint maps bit-exact; one operator apply and the
operator diagonal within 1e-12 relative L2; fields after N explicit steps within 1e-9; the
GMG-preconditioned CG solution within 1e-8 with an iteration count within 10 % (or 2)."""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def load(name):
    return np.load(GOLDEN / f"{name}.npz")


def test_allen_cahn_golden(gpu_lib):
    g = load("allen_cahn_2d_q2")
    wl = G.wl_allen_cahn()
    assert np.array_equal(wl.initial[0], g["n0"])
    p = wl.make_problem()
    assert np.array_equal(p.dof_map(0), g["dof_map"])
    assert rel_l2(p.invm(), g["invm"]) < 1e-14
    p.upload(0, g["n0"], age=1)
    assert rel_l2(p.apply(0, 0, None, scale=1), g["rhs_apply"]) < 1e-12
    p.close()
    p = wl.make_problem()
    p.solve(25, output_every=25)
    assert rel_l2(p.download(0, age=1), g["n_25"]) < 1e-9
    assert rel_l2(p.download(1), g["mg_n_25"]) < 1e-9
    assert rel_l2(p.download(2), g["f_tot_25"]) < 1e-9


def test_cahn_hilliard_golden(gpu_lib):
    g = load("cahn_hilliard_3d_q2")
    wl = G.wl_cahn_hilliard()
    p = wl.make_problem()
    cm = p.constraint_map(0).astype(np.int64)
    ref = g["cmap"]
    assert np.array_equal(cm[ref >= 0], ref[ref >= 0]) and np.array_equal(cm >= 0, ref >= 0)
    p.solve(10)
    assert rel_l2(p.download(0, age=1), g["c_10"]) < 1e-9
    assert rel_l2(p.download(1, age=1), g["mu_10"]) < 1e-9


def test_coupled_golden(gpu_lib):
    g = load("coupled_acch_2d_q2")
    p = G.wl_coupled().make_problem()
    p.solve(12, output_every=6)
    for f, key, age in ((0, "c_12", 1), (1, "n_12", 1), (2, "f_tot_12", 0), (3, "mag_grad_c_12", 0)):
        assert rel_l2(p.download(f, age=age), g[key]) < 1e-9, key


def test_elasticity_golden(gpu_lib):
    g = load("elasticity_3d_q2")
    wl = G.wl_elasticity()
    p = wl.make_problem()
    assert np.array_equal(p.dof_map(1), g["vector_dof_map"])
    cm = p.constraint_map(0).astype(np.int64)
    ref = g["cmap"]
    assert np.array_equal(cm >= 0, ref >= 0) and np.array_equal(cm[ref >= 0], ref[ref >= 0])
    assert rel_l2(p.apply(0, 1, g["src"], scale=0), g["lhs_apply"]) < 1e-12
    assert rel_l2(p.apply(0, 0, None, scale=0), g["rhs_apply"]) < 1e-12
    p.set_linear_params(0, **G.ELASTICITY_SOLVER)
    assert rel_l2(p.lhs_diagonal(0), g["diagonal"]) < 1e-12
    its, res = p.linear_solve(0)
    assert res < 1e-11
    assert abs(its - int(g["iterations"])) <= max(2, 0.1 * int(g["iterations"]))
    assert rel_l2(p.download(0), g["u"]) < 1e-8


def test_allen_cahn_adaptive_golden(gpu_lib):
    g = load("allen_cahn_amr_2d_q2")
    wl = G.wl_allen_cahn_amr()
    assert np.array_equal(wl.initial[0], g["n0"])
    p = wl.make_problem()
    p.solve(12, output_every=12)
    assert np.array_equal(p.cells().astype(np.int64), g["cells"])
    assert np.array_equal(p.cell_dofs().astype(np.int64), g["cell_dofs"])
    cnt, mas, w = p.hanging()
    assert np.array_equal(cnt, g["hang_count"]) and np.array_equal(mas, g["hang_master"])
    assert np.array_equal(w, g["hang_weight"])
    assert rel_l2(p.invm(), g["invm"]) < 1e-14
    assert rel_l2(p.download(0, 1, 2), g["n_12"]) < 1e-9
    assert rel_l2(p.download(1, 0, 2), g["mg_n_12"]) < 1e-9
    assert rel_l2(p.download(2, 0, 2), g["f_tot_12"]) < 1e-9

