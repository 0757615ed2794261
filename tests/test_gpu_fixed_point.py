"""The exact fixed-point contractions of the FP64 Q1/Q2 cell kernels (64-bit integer derivative
and integration sums with a per-cell block exponent, include/prismspf/gpu/fixed_point.cuh)
against the oracle and against the same kernels contracting in FP64.

Bars: one operator apply within 1e-12 relative L2 of the oracle (the FP64 apply bar), in every
mode (1 integer derivatives + FP64 integration, 2 both integer, 3 FP64 derivatives + integer
integration), non-cubic cells, fields scaled far from O(1) and values spanning many
binades inside a cell; fixed point against FP64 contractions within 1e-13 relative L2 (both
are FP64-accurate; their difference is rounding)."""
import contextlib
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu

APPLY_TOL = 1e-12


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@contextlib.contextmanager
def env(**kw):
    old = {k: os.environ.get(k) for k in kw}
    os.environ.update({k: v for k, v in kw.items()})
    try:
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def ch_problem(dim, degree, size=None, scale_c=1.0, scale_mu=1.0, seed=3):
    wl = W.cahn_hilliard_3d(refine=2 if dim == 3 else 4, degree=degree, dim=dim, size=8.0)
    if size is not None:
        wl.mesh.size = size
    p = wl.make_problem()
    o = po.Oracle(wl)
    rng = np.random.default_rng(seed)
    N = p.n_nodes
    c = wl.initial[0] * scale_c
    mu = rng.uniform(-1, 1, N) * scale_mu
    for f, v in ((0, c), (1, mu)):
        p.upload(f, v, age=1)
        o.set(f, v, age=1)
    p.upload(0, c, age=0)
    o.set(0, c, age=0)
    return p, o


MODES = ["1", "2", "3", "4"]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dim,degree", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_apply_matches_oracle_in_every_mode(gpu_lib, dim, degree, mode):
    with env(PPF_CONTRACTION_MODE=mode):
        p, o = ch_problem(dim, degree)
        for b in (0, 1):
            got = p.apply(b, 0, None, scale=1)
            ref = o.apply(b, 0, None, scale=1)
            assert rel_l2(got, ref) < APPLY_TOL, b
            assert p.contraction_mode(b, 0) == int(mode)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dim", [2, 3])
def test_non_cubic_cells(gpu_lib, dim, mode):
    """h_x != h_y (!= h_z): per-direction derivative scales, per-direction integration scales."""
    size = (8.0, 5.0, 3.0) if dim == 3 else (8.0, 3.0, 1.0)
    with env(PPF_CONTRACTION_MODE=mode):
        p, o = ch_problem(dim, 2, size=size)
        for b in (0, 1):
            got = p.apply(b, 0, None, scale=1)
            ref = o.apply(b, 0, None, scale=1)
            assert rel_l2(got, ref) < APPLY_TOL, b
            assert p.contraction_mode(b, 0) == (1 if mode == "4" else int(mode))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("scale", [1e-150, 1e-20, 1e20, 1e150])
def test_fields_far_from_unit_scale(gpu_lib, scale, mode):
    """The c block is linear in (c, mu): scaling both moves every block exponent."""
    with env(PPF_CONTRACTION_MODE=mode):
        p, o = ch_problem(3, 2, scale_c=scale, scale_mu=scale)
        got = p.apply(0, 0, None, scale=1)
        ref = o.apply(0, 0, None, scale=1)
        assert np.all(np.isfinite(got))
        assert rel_l2(got, ref) < APPLY_TOL


@pytest.mark.parametrize("mode", MODES)
def test_values_spanning_many_binades_in_a_cell(gpu_lib, mode):
    """mu = U(-1, 1) * 10^U(-30, 0) per node: small values share a cell with large ones."""
    wl = W.cahn_hilliard_3d(refine=2, degree=2, dim=3, size=8.0)
    with env(PPF_CONTRACTION_MODE=mode):
        p = wl.make_problem()
        o = po.Oracle(wl)
        rng = np.random.default_rng(9)
        N = p.n_nodes
        mu = rng.uniform(-1, 1, N) * 10.0 ** rng.uniform(-30, 0, N)
        c = wl.initial[0]
        for f, v in ((0, c), (1, mu)):
            p.upload(f, v, age=1)
            o.set(f, v, age=1)
        got = p.apply(0, 0, None, scale=1)
        ref = o.apply(0, 0, None, scale=1)
        assert rel_l2(got, ref) < APPLY_TOL


@pytest.mark.parametrize("mode", MODES)
def test_vector_elasticity_lhs(gpu_lib, mode):
    """Symmetric gradients of a vector field and a tensor gradient term (3 components)."""
    wl = W.eshelby_3d(refine=2, degree=2, size=16.0, n_incl=5, dim=3)
    with env(PPF_CONTRACTION_MODE=mode):
        p = wl.make_problem()
        o = po.Oracle(wl)
        u = np.random.default_rng(11).uniform(-1, 1, p.field_length(0))
        got = p.apply(0, 1, u, scale=0)
        ref = o.apply(0, 1, u, scale=0)
        assert rel_l2(got, ref) < APPLY_TOL
        assert p.contraction_mode(0, 1) == int(mode)


def test_fixed_point_against_fp64_contractions(gpu_lib):
    """Every mode against FP64 contractions on the same inputs."""
    outs = {}
    for key, kw in (("0", {"PPF_FP64_CONTRACTIONS": "1"}), ("1", {"PPF_CONTRACTION_MODE": "1"}),
                    ("2", {"PPF_CONTRACTION_MODE": "2"}), ("3", {"PPF_CONTRACTION_MODE": "3"}),
                    ("4", {"PPF_CONTRACTION_MODE": "4"})):
        with env(**kw):
            p, _ = ch_problem(3, 2)
            outs[key] = [p.apply(b, 0, None, scale=1) for b in (0, 1)]
            assert p.contraction_mode(0, 0) == int(key)
    for key in ("1", "2", "3", "4"):
        for b in (0, 1):
            assert rel_l2(outs[key][b], outs["0"][b]) < 1e-13, (key, b)


def test_modes_outside_the_fixed_point_path(gpu_lib):
    wl = W.allen_cahn_2d(refine=3, degree=3)
    p = wl.make_problem()
    p.upload(0, wl.initial[0], age=1)
    p.apply(0, 0, None, scale=1)
    assert p.contraction_mode(0, 0) == 0  # Q3: FP64 contractions
    wl = W.allen_cahn_2d(refine=3, degree=2)
    p = wl.make_problem()
    p.upload(0, wl.initial[0], age=1)
    p.apply(0, 0, None, scale=1)
    assert p.contraction_mode(0, 0) in (1, 2, 3, 4)  # chosen by timing the modes on the first launch


@pytest.mark.parametrize("mode", MODES)
def test_nonfinite_value_reports_nan_in_every_mode(gpu_lib, mode):
    """A NaN in a gradient row gives its cell block exponent 2047: the cell's derivatives (and
    integer integration) return NaN and the finalize kernel reports PPF_ERR_NAN."""
    from phasefield_gb300 import capi
    wl = W.cahn_hilliard_3d(refine=2, degree=2, dim=3, size=8.0, dt=1e-4)
    with env(PPF_CONTRACTION_MODE=mode):
        p = wl.make_problem()
        p.solve(0)
        mu = p.download(1, age=1)
        mu[len(mu) // 2] = np.nan
        p.upload(1, mu, age=1)
        with pytest.raises(capi.PPFError) as e:
            p.solve(1)
        assert e.value.code == capi.PPF_ERR_NAN


@pytest.mark.parametrize("mode", ["1", "2", "4"])
def test_derivative_error_is_absolute_in_the_cell_maximum(gpu_lib, mode):
    """Per entry, a derivative taken in fixed point is exact to the block resolution of its
    cell: the absolute error is at most (sum of |D| over the line) x 2^(e - 58) / h, e the
    binary exponent of the cell's largest value, plus the final rounding. Every Q2 cell here
    holds O(1) corner values and an O(1e-12) cross through its centre, so the gradient at the
    centre node is O(1e-13) while the cell's block exponent is that of its O(1) corners: there
    the error stays within the absolute bound (a relative error of order 1e-6 of the small
    gradient itself), while FP64 contractions of the same line keep 1e-13 relative. The
    post-processing block's |grad n| at each cell's centre node (interior to one cell, so the
    lumped-mass scaling returns the point value) exposes the derivative itself. In mode 4 (the
    lane kernel) the value term |grad n| is integrated in fixed point too, with the block exponent
    of the cell's largest submitted term: one more unit of 2^-52 of that term."""
    wl = W.allen_cahn_2d(refine=3, degree=2)  # 8 x 8 Q2 cells of [0,100]^2, 17 x 17 nodes
    nc, nn, h = 8, 17, 100.0 / 8
    rng = np.random.default_rng(23)
    u = rng.uniform(0.5, 1.0, (nn, nn))  # [y, x]
    small = 1e-12
    for c in range(nc):  # the row and column through every cell centre
        u[2 * c + 1, :] = small * rng.uniform(-1, 1, nn)
        u[:, 2 * c + 1] = small * rng.uniform(-1, 1, nn)
    n0 = u.ravel()
    centre = np.array([(2 * cy + 1) * nn + 2 * cx + 1 for cy in range(nc) for cx in range(nc)])
    # the exact centre gradients of the quadratic interpolant: (u_right - u_left) / h per direction
    gx = np.array([(u[2 * cy + 1, 2 * cx + 2] - u[2 * cy + 1, 2 * cx]) / h for cy in range(nc) for cx in range(nc)])
    gy = np.array([(u[2 * cy + 2, 2 * cx + 1] - u[2 * cy, 2 * cx + 1]) / h for cy in range(nc) for cx in range(nc)])
    exact = np.hypot(gx, gy)
    cell_max = np.array([np.abs(u[2 * cy:2 * cy + 3, 2 * cx:2 * cx + 3]).max() for cy in range(nc) for cx in range(nc)])
    resolution = 2.0 ** (np.floor(np.log2(cell_max)) - 58)

    def centre_gradients(**kw):
        with env(**kw):
            p = wl.make_problem()
            p.upload(0, n0, age=0)
            out = p.apply(1, 0, None, scale=1)  # the post-processing block: mg_n, then f_tot
            p.close()
        return out[:nn * nn][centre]

    fp64 = centre_gradients(PPF_FP64_CONTRACTIONS="1")
    assert np.all(np.abs(fp64 - exact) <= 1e-13 * exact)
    fixed = centre_gradients(PPF_CONTRACTION_MODE=mode)
    bound = 2.0 * np.sqrt(2.0) * resolution / h + 8 * np.spacing(exact)
    if mode == "4":
        # the lane kernel integrates the value terms in fixed point as well, as h |grad n| with
        # the block exponent of the cell's largest one (one binade up, h = 12.5 not being a power
        # of two): one unit of that resolution more, relative to the cell's largest |grad n|
        D = np.array([[-3.0, 4.0, -1.0], [-1.0, 0.0, 1.0], [1.0, -4.0, 3.0]]) / h
        gmax = np.array([np.hypot(u[2 * cy:2 * cy + 3, 2 * cx:2 * cx + 3] @ D.T,
                                  D @ u[2 * cy:2 * cy + 3, 2 * cx:2 * cx + 3]).max()
                         for cy in range(nc) for cx in range(nc)])
        hk = np.floor(np.log2(h))
        bound = bound + 2.0 ** (np.floor(np.log2(gmax)) + hk + 1 - 52) / h
    assert np.all(np.abs(fixed - exact) <= bound)


@pytest.mark.parametrize("dim,degree,sub", [(3, 2, (3, 1, 2)), (3, 1, (5, 3, 1)), (2, 2, (3, 5, 1)), (2, 1, (7, 3, 1))])
def test_lane_kernel_partial_tiles(gpu_lib, dim, degree, sub):
    """The lane kernel on lattices of square cells whose cell count is not a multiple of its
    32-cell tile (the last tile's spare lanes recompute the last cell and scatter nothing), with
    different cell counts per direction: both blocks' applies and five steps against the oracle."""
    size = 4.0 * np.array(sub[:dim], dtype=float)
    wl = W.cahn_hilliard_3d(refine=1 if dim == 3 else 2, degree=degree, dim=dim, size=1.0, subdivisions=sub[:dim] + (1,) * (3 - dim))
    wl.mesh.size = tuple(size) + (1.0,) * (3 - dim)
    with env(PPF_CONTRACTION_MODE="4"):
        p = wl.make_problem()
        o = po.Oracle(wl)
        assert p.n_cells % 32 != 0
        rng = np.random.default_rng(17)
        mu = rng.uniform(-1, 1, p.n_nodes)
        for f, v in ((0, wl.initial[0]), (1, mu)):
            p.upload(f, v, age=1)
            o.set(f, v, age=1)
        p.upload(0, wl.initial[0], age=0)
        o.set(0, wl.initial[0], age=0)
        for b in (0, 1):
            got = p.apply(b, 0, None, scale=1)
            ref = o.apply(b, 0, None, scale=1)
            assert rel_l2(got, ref) < APPLY_TOL, b
            assert p.contraction_mode(b, 0) == 4
        p.close()
        p = wl.make_problem()
        p.solve(5)
        o = po.Oracle(wl)
        assert o.run(5) == 0
        for f in (0, 1):
            assert rel_l2(p.download(f, age=1), o.get(f, 1)) < 1e-9, f
