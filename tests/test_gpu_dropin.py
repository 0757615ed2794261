"""GPU tests of the drop-in application path: an application written against the reference's
C++ API (examples/*: main.cc + custom_pde.h + a parameter file) is compiled with nvcc, run on
the GPU, and its VTU output is checked against the oracle.

The initial condition is read back from the application's increment-0 output (its values at
the support points: the output patches of degree <= 2 elements put their points on the
Gauss-Lobatto nodes), handed to the oracle, and the oracle's fields after the same increments
are compared with the application's final output.
Bars: explicit runs within 1e-9 relative L2 (as the engine's own step tests); the linear
elasticity solve within 1e-8 relative L2 (both solvers stop at the same absolute residual).
"""
import re
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
EXAMPLES = ROOT / "examples"


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def read_vtu(path: Path) -> dict:
    """Points and point-data arrays of a raw-appended VTU file as written by the drop-in."""
    raw = path.read_bytes()
    head_end = raw.index(b"<AppendedData")
    header = raw[:head_end].decode()
    start = raw.index(b"_", head_end) + 1
    arrays = {}
    for m in re.finditer(r'<DataArray type="(\w+)"(?: Name="([^"]*)")?(?: NumberOfComponents="(\d+)")?'
                         r'(?: NumberOfTuples="\d+")? format="appended" offset="(\d+)"', header):
        typ, name, ncomp, off = m.group(1), m.group(2) or "Points", int(m.group(3) or 1), int(m.group(4))
        nbytes = struct.unpack_from("<Q", raw, start + off)[0]
        dt = {"Float64": "<f8", "Int64": "<i8", "UInt8": "u1"}[typ]
        a = np.frombuffer(raw, dtype=dt, count=nbytes // np.dtype(dt).itemsize, offset=start + off + 8)
        arrays[name] = a.reshape(-1, ncomp) if ncomp > 1 else a
    return arrays


def to_lattice(vtu: dict, mesh, name: str, ncomp: int = 1) -> np.ndarray:
    """Point values of a field placed on the lattice (lattice order, component-major)."""
    pts = vtu["Points"]
    k = mesh.degree
    idx = np.zeros(len(pts), dtype=np.int64)
    stride = 1
    for d in range(mesh.dim):
        h = mesh.size[d] / mesh.cells[d]
        i = np.rint((pts[:, d] - mesh.lower[d]) / h * k).astype(np.int64)
        idx += i * stride
        stride *= mesh.nodes[d]
    N = int(np.prod(mesh.nodes))
    vals = vtu[name]
    out = np.full(ncomp * N, np.nan)
    for c in range(ncomp):
        out[c * N + idx] = vals if ncomp == 1 else vals[:, c]
    assert not np.isnan(out).any(), "every lattice node appears in the output"
    return out


def build_and_run(app: str, prm_text: str, tmp_path: Path):
    from phasefield_gb300 import app_build
    exe = app_build.compile_app(EXAMPLES / app, tmp_path / app)
    (tmp_path / "parameters.prm").write_text(prm_text)
    r = subprocess.run([str(exe), "-i", "parameters.prm"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def logged_norms(stdout: str, increment: int) -> dict:
    block = stdout.split(f"Iteration {increment} Time")[1].split("\n\n")[0]
    return {m.group(1): float(m.group(2)) for m in re.finditer(r"name (\S+) l2-norm (\S+)", block)}


def test_allen_cahn_application_matches_oracle(gpu_lib, tmp_path):
    n = 50
    out = build_and_run("allen_cahn_explicit", f"""
set global refinement = 5
subsection Rectangular mesh
  set x size = 100.0
  set y size = 100.0
end
set time step = 0.01
set number steps = {n}
subsection output
  set number = 1
end
subsection miscellaneous
  set random seed = 99
end
set Model constant mobility = 1.0, DOUBLE
set Model constant kappa = 2.0, DOUBLE
set Model constant n_grains = 12, INT
""", tmp_path)
    wl = W.allen_cahn_2d(refine=5, degree=1, dt=0.01)
    v0 = read_vtu(tmp_path / "solutions" / "solution_00.vtu")
    n0 = to_lattice(v0, wl.mesh, "n")
    assert 0.5 < n0.max() <= 1.0 and n0.min() >= 0.0  # seeded grains
    wl.initial = {0: n0}
    o = po.Oracle(wl)
    assert o.run(n, n) == 0
    v1 = read_vtu(tmp_path / "solutions" / f"solution_{n}.vtu")
    assert rel_l2(to_lattice(v1, wl.mesh, "n"), o.get(0, 1)) < 1e-9
    for f, name in ((1, "mg_n"), (2, "f_tot")):
        assert rel_l2(to_lattice(v1, wl.mesh, name), o.get(f, 0)) < 1e-9, name
    norms = logged_norms(out, n)  # printed with the stream's default 6 significant digits
    assert norms["n"] == pytest.approx(np.linalg.norm(o.get(0, 1)), rel=1e-5)


def test_cahn_hilliard_application_matches_oracle(gpu_lib, tmp_path):
    n = 30
    build_and_run("cahn_hilliard_explicit", f"""
set global refinement = 2
subsection Rectangular mesh
  set x size = 4.0
  set y size = 4.0
  set z size = 4.0
  set x periodic = true
  set y periodic = true
  set z periodic = true
end
set time step = 1.0e-4
set number steps = {n}
subsection output
  set number = 1
end
set Model constant mobility = 1.0, DOUBLE
set Model constant kappa = 1.5, DOUBLE
set Model constant well_height = 4.0, DOUBLE
set Model constant c0 = 0.5, DOUBLE
set Model constant amplitude = 0.05, DOUBLE
""", tmp_path)
    wl = W.cahn_hilliard_3d(refine=2, degree=2, size=4.0, dt=1e-4)
    v0 = read_vtu(tmp_path / "solutions" / "solution_00.vtu")
    c0 = to_lattice(v0, wl.mesh, "c")
    assert np.all(np.abs(c0 - 0.5) <= 0.05)
    wl.initial = {0: c0}
    o = po.Oracle(wl)
    assert o.run(n, n) == 0
    v1 = read_vtu(tmp_path / "solutions" / f"solution_{n}.vtu")
    for f, name, age in ((0, "c", 1), (1, "mu", 1), (2, "f_tot", 0)):
        assert rel_l2(to_lattice(v1, wl.mesh, name), o.get(f, age)) < 1e-9, name


def test_eshelby_application_matches_oracle(gpu_lib, tmp_path):
    incl = [(4.0, 5.0, 7.5, 2.5), (10.0, 11.0, 6.0, 2.0), (12.0, 4.0, 12.0, 3.0)]
    consts = "\n".join(f"set Model constant inclusion_{i} = ({x}, {y}, {z}), TENSOR\n"
                       f"set Model constant radius_{i} = {r}, DOUBLE" for i, (x, y, z, r) in enumerate(incl))
    build_and_run("eshelby_inclusion", f"""
set global refinement = 2
subsection Rectangular mesh
  set x size = 16.0
  set y size = 16.0
  set z size = 16.0
end
subsection boundary conditions: 0
  set variables = u
  set conditions = Dirichlet, Natural, Natural, Natural, Natural, Natural
end
subsection linear solver parameters: 0
  set solver_ids = 1
  set tolerance type = AbsoluteResidual
  set tolerance value = 1e-10
  set max iterations = 1000
  set preconditioner type = GMG
  set mg depth = 3
  subsection Chebyshev
    set smoother degree = 4
  end
end
set Model constant stiffness = (250, 250, 250, 100, 100, 100, 150, 150, 0, 0, 0, 150, 0, 0, 0, 0, 0, 0, 0, 0, 0), anisotropic elastic constants
set Model constant eigenstrain = 0.01, DOUBLE
set Model constant interface_width = 1.0, DOUBLE
set Model constant n_inclusions = {len(incl)}, INT
{consts}
""", tmp_path)
    wl = W.eshelby_3d(refine=2, degree=2, size=16.0, n_incl=len(incl))
    C = W.cubic_stiffness(250.0, 150.0, 100.0)
    wl.constants = list(C.ravel()) + [0.01, 1.0, float(len(incl))] + [v for t in incl for v in t]
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=0, tolerance=1e-10, max_iterations=1000, preconditioner=2, mg_depth=3,
                        smoother_degree=4)
    assert o.run(0) == 0
    v = read_vtu(tmp_path / "solutions" / "solution_0.vtu")
    u = to_lattice(v, wl.mesh, "u", ncomp=3)
    assert np.abs(u).max() > 1e-4  # the inclusions load the body
    assert rel_l2(u, o.get(0, 0)) < 1e-8


def test_implicit_allen_cahn_application_matches_oracle(gpu_lib, tmp_path):
    """A Newton block through the drop-in: the application's linear/Newton parameters reach the
    engine by solve-block id and the implicit steps match the oracle's Newton solver."""
    n = 6
    build_and_run("allen_cahn_implicit", f"""
set global refinement = 4
subsection Rectangular mesh
  set x size = 100.0
  set y size = 100.0
end
set time step = 1.0
set number steps = {n}
subsection output
  set number = 1
end
subsection linear solver parameters: 0
  set solver_ids = 1
  set tolerance type = RMSEPerField
  set tolerance value = 1e-13
  set max iterations = 3000
end
subsection newton solver parameters: 0
  set solver_ids = 1
  set max iterations = 50
  set tolerance value = 1e-12
end
subsection miscellaneous
  set random seed = 7
end
set Model constant mobility = 1.0, DOUBLE
set Model constant kappa = 2.0, DOUBLE
set Model constant n_grains = 12, INT
""", tmp_path)
    wl = W.allen_cahn_implicit_2d(refine=4, dt=1.0)
    v0 = read_vtu(tmp_path / "solutions" / "solution_0.vtu")
    wl.initial = {0: to_lattice(v0, wl.mesh, "n")}
    o = po.Oracle(wl)
    o.set_linear_params(0, tolerance_type=1, tolerance=1e-13, max_iterations=3000)
    o.set_newton_params(0, max_iterations=50, tolerance=1e-12)
    assert o.run(n, n) == 0
    v1 = read_vtu(tmp_path / "solutions" / f"solution_{n}.vtu")
    assert rel_l2(to_lattice(v1, wl.mesh, "n"), o.get(0, 1)) < 1e-8
    assert rel_l2(to_lattice(v1, wl.mesh, "f_tot"), o.get(2, 0)) < 1e-8


@pytest.mark.parametrize("mode", [None, "4"])
def test_derivative_getters_are_exact_on_quadratics(gpu_lib, tmp_path, monkeypatch, mode):
    """Hessian, Hessian diagonal, Laplacian, divergence, curl, symmetric gradient, quadrature
    point and element volume through the drop-in, on inputs FE_Q(2) represents exactly (two
    post-processing blocks); with the contraction mode timed, and fixed to the lane kernel (mode
    4: its row layout for values, Hessians and gradients)."""
    from phasefield_gb300 import app_build
    if mode:
        monkeypatch.setenv("PPF_CONTRACTION_MODE", mode)
    src = ROOT / "tests" / "dropin" / "derivatives"
    exe = app_build.compile_app(src, tmp_path / "derivatives")
    (tmp_path / "parameters.prm").write_text("""
set global refinement = 2
subsection Rectangular mesh
  set x size = 2.0
  set y size = 2.0
end
set number steps = 0
""")
    r = subprocess.run([str(exe), "-i", "parameters.prm"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    v = read_vtu(tmp_path / "solutions" / "solution_0.vtu")
    x, y = v["Points"][:, 0], v["Points"][:, 1]
    vol = (2.0 / 4) ** 2
    expect = {"lap_u": 6.0 + 0 * x, "hess_u": 531.0 + 0 * x, "div_w": 3.0 * x, "curl_w": y - 1.0,
              "sym_w_xy": 0.5 * (1.0 + y), "x_plus_vol": x + vol}
    for name, ref in expect.items():
        assert np.abs(v[name] - ref).max() < 1e-10, name


def test_allen_cahn_application_on_an_adaptive_mesh_matches_oracle(gpu_lib, tmp_path):
    """`mesh adaptivity = true` with the reference application's criterion (0.01 < n < 0.99):
    the initial condition comes from a uniform run of the same application at increment 0, the
    oracle refines, steps and remeshes from it, and the adaptive run's output patches must carry
    the oracle's values at their points."""
    common = """
subsection Rectangular mesh
  set x size = 100.0
  set y size = 100.0
end
set time step = 0.01
subsection miscellaneous
  set random seed = 99
end
set Model constant mobility = 1.0, DOUBLE
set Model constant kappa = 2.0, DOUBLE
set Model constant n_grains = 12, INT
"""
    n = 30
    uni = tmp_path / "uniform"
    uni.mkdir()
    build_and_run("allen_cahn_explicit", "set global refinement = 5\nset number steps = 0\n" + common, uni)
    wl = W.allen_cahn_amr_2d(refine=5, degree=1, min_level=3, max_level=6, period=10, dt=0.01)
    wl.initial = {0: to_lattice(read_vtu(uni / "solutions" / "solution_0.vtu"), wl.mesh, "n")}
    ada = tmp_path / "adaptive"
    ada.mkdir()
    out = build_and_run("allen_cahn_explicit", f"""
set global refinement = 5
set max refinement = 6
set min refinement = 3
set mesh adaptivity = true
set remeshing period = 10
subsection refinement criterion: 0
  set type = value
  set value lower bound = 0.01
  set value upper bound = 0.99
  set variables = n
end
set number steps = {n}
subsection output
  set number = 1
end
""" + common, ada)
    assert "not applied" not in out
    o = po.Oracle(wl, adaptivity=wl.adaptivity)
    assert o.run(n, n) == 0
    assert len(np.unique(o.cells()[:, 0])) > 1
    v = read_vtu(ada / "solutions" / f"solution_{n}.vtu")
    idx = oracle_points(v, o, wl)
    assert rel_l2(v["n"], o.get_native(0, 1)[idx]) < 1e-9
    for f, name in ((1, "mg_n"), (2, "f_tot")):
        assert rel_l2(v[name], o.get_native(f, 0)[idx]) < 1e-9, name
    norms = logged_norms(out, n)
    assert norms["n"] == pytest.approx(np.linalg.norm(o.get_native(0, 1)), rel=1e-5)


def oracle_points(v: dict, o, wl) -> np.ndarray:
    """For the points of an adaptive run's output patches (one patch of (degree+1)^dim points
    per active cell of the oracle's mesh, on the Gauss-Lobatto nodes for degrees 1 and 2), the
    oracle DoF at the same position."""
    dim, k = wl.mesh.dim, wl.mesh.degree
    assert len(v["Points"]) == (k + 1) ** dim * o.n_cells()
    h_min = wl.mesh.size[0] / (wl.mesh.subdivisions[0] << wl.adaptivity["max_level"]) / k
    ext = np.array([int(round(wl.mesh.size[d] / h_min)) for d in range(dim)])
    per = np.array([bool(wl.mesh.periodic[d]) for d in range(dim)])

    def key(x):  # node units; periodic images wrap onto their master, as the DoFs do
        i = np.rint(x[:, :dim] / h_min).astype(np.int64)
        i = np.where(per, i % ext, i)
        return tuple(i.T)

    where = {k: i for i, k in enumerate(zip(*key(o.node_points())))}
    return np.array([where[k] for k in zip(*key(v["Points"]))])


def test_implicit_allen_cahn_application_on_an_adaptive_mesh_matches_oracle(gpu_lib, tmp_path):
    """Newton blocks on an adaptive mesh through the drop-in (no preconditioner, remeshing every
    2 increments), against the oracle started from the same initial condition."""
    common = """
subsection Rectangular mesh
  set x size = 100.0
  set y size = 100.0
end
set time step = 1.0
subsection linear solver parameters: 0
  set solver_ids = 1
  set tolerance type = RMSEPerField
  set tolerance value = 1e-13
  set max iterations = 3000
end
subsection newton solver parameters: 0
  set solver_ids = 1
  set max iterations = 50
  set tolerance value = 1e-12
end
subsection miscellaneous
  set random seed = 7
end
set Model constant mobility = 1.0, DOUBLE
set Model constant kappa = 2.0, DOUBLE
set Model constant n_grains = 12, INT
"""
    n = 6
    uni = tmp_path / "uniform"
    uni.mkdir()
    build_and_run("allen_cahn_implicit", "set global refinement = 4\nset number steps = 0\n" + common, uni)
    wl = W.allen_cahn_implicit_2d(refine=4, dt=1.0)
    wl.adaptivity = dict(min_level=3, max_level=6, period=2, criteria=[(0, 1, 0.01, 0.99, 0.0)])
    wl.initial = {0: to_lattice(read_vtu(uni / "solutions" / "solution_0.vtu"), wl.mesh, "n")}
    ada = tmp_path / "adaptive"
    ada.mkdir()
    out = build_and_run("allen_cahn_implicit", f"""
set global refinement = 4
set max refinement = 6
set min refinement = 3
set mesh adaptivity = true
set remeshing period = 2
subsection refinement criterion: 0
  set type = value
  set value lower bound = 0.01
  set value upper bound = 0.99
  set variables = n
end
set number steps = {n}
subsection output
  set number = 1
end
""" + common, ada)
    assert "not applied" not in out
    o = po.Oracle(wl, adaptivity=wl.adaptivity)
    o.set_linear_params(0, tolerance_type=1, tolerance=1e-13, max_iterations=3000)
    o.set_newton_params(0, max_iterations=50, tolerance=1e-12)
    assert o.run(n, n) == 0
    assert len(np.unique(o.cells()[:, 0])) > 1
    v = read_vtu(ada / "solutions" / f"solution_{n}.vtu")
    idx = oracle_points(v, o, wl)
    assert rel_l2(v["n"], o.get_native(0, 1)[idx]) < 1e-8
    assert rel_l2(v["f_tot"], o.get_native(2, 0)[idx]) < 1e-8


def test_cahn_hilliard_application_on_a_3d_adaptive_mesh_matches_oracle(gpu_lib, tmp_path):
    """The periodic 3-D Cahn-Hilliard application (Q2) with a gradient criterion: hanging nodes
    on faces and edges, periodic images, and the 3-D output of an adaptive mesh."""
    common = """
subsection Rectangular mesh
  set x size = 4.0
  set y size = 4.0
  set z size = 4.0
  set x periodic = true
  set y periodic = true
  set z periodic = true
end
set time step = 2.0e-5
set Model constant mobility = 1.0, DOUBLE
set Model constant kappa = 1.5, DOUBLE
set Model constant well_height = 4.0, DOUBLE
set Model constant c0 = 0.5, DOUBLE
set Model constant amplitude = 0.05, DOUBLE
"""
    n = 10
    uni = tmp_path / "uniform"
    uni.mkdir()
    build_and_run("cahn_hilliard_explicit", "set global refinement = 2\nset number steps = 0\n" + common, uni)
    wl = W.cahn_hilliard_3d(refine=2, degree=2, size=4.0, dt=2e-5)
    wl.adaptivity = dict(min_level=1, max_level=3, period=5, criteria=[(0, 2, 0.0, 0.0, 0.18)])
    wl.initial = {0: to_lattice(read_vtu(uni / "solutions" / "solution_0.vtu"), wl.mesh, "c")}
    ada = tmp_path / "adaptive"
    ada.mkdir()
    out = build_and_run("cahn_hilliard_explicit", f"""
set global refinement = 2
set max refinement = 3
set min refinement = 1
set mesh adaptivity = true
set remeshing period = 5
subsection refinement criterion: 0
  set type = gradient
  set gradient magnitude lower bound = 0.18
  set variables = c
end
set number steps = {n}
subsection output
  set number = 1
end
""" + common, ada)
    assert "not applied" not in out
    o = po.Oracle(wl, adaptivity=wl.adaptivity)
    assert o.run(n, n) == 0
    assert len(np.unique(o.cells()[:, 0])) > 1
    v = read_vtu(ada / "solutions" / f"solution_{n}.vtu")
    idx = oracle_points(v, o, wl)
    for f, name, age in ((0, "c", 1), (1, "mu", 1), (2, "f_tot", 0)):
        assert rel_l2(v[name], o.get_native(f, age)[idx]) < 1e-9, name

