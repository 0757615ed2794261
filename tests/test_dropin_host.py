"""CPU tests of the drop-in C++ host layer (include/prismspf/...): the reference's application
sources compile unchanged against it, its parameter-file reader follows the reference's
entries, aliases and defaults, and make_dependency_set parses the dependency grammar like the
reference (include/prismspf/core/dependencies.h:134-213).

Compile-only on this machine: nvcc cross-compiles the device code without a GPU.
"""
import json
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"
EXAMPLES = ROOT / "examples"
# the reference tree (read only by these CPU checks); PPF_REFERENCE_ROOT points elsewhere
REF_APPS = Path(os.environ.get("PPF_REFERENCE_ROOT", "/root/reference")) / "applications"
GXX = shutil.which("g++")
NVCC = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)

needs_gxx = pytest.mark.skipif(GXX is None, reason="g++ not available")
needs_ref = pytest.mark.skipif(not REF_APPS.is_dir(), reason="reference sources not present")


def host_syntax(app_dir: Path):
    r = subprocess.run([GXX, "-std=c++20", "-fsyntax-only", "-I", str(INCLUDE), "-I", str(app_dir),
                        str(app_dir / "main.cc")], capture_output=True, text=True)
    return r.returncode, r.stderr


@pytest.fixture(scope="session")
def prm_dump(tmp_path_factory):
    if GXX is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("prm") / "prm_dump"
    r = subprocess.run([GXX, "-std=c++20", "-O1", "-I", str(INCLUDE), str(ROOT / "tests/dropin/prm_dump.cc"), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(dim, text=None, path=None, tmp=tmp_path_factory.mktemp("prmfiles")):
        if text is not None:
            path = tmp / f"p{abs(hash(text))}.prm"
            path.write_text(text)
        out = subprocess.run([str(exe), str(dim), str(path)], capture_output=True, text=True, check=True).stdout
        return json.loads(out)

    run.exe = exe
    return run


# ---------------------------------------------------------------------------------------------
# sources compile unchanged
# ---------------------------------------------------------------------------------------------
@needs_gxx
@pytest.mark.parametrize("app", ["allen_cahn_explicit", "allen_cahn_implicit", "cahn_hilliard_explicit",
                                 "eshelby_inclusion"])
def test_example_apps_host_syntax(app):
    rc, err = host_syntax(EXAMPLES / app)
    assert rc == 0, err


@needs_gxx
def test_derivative_test_app_host_syntax():
    rc, err = host_syntax(ROOT / "tests" / "dropin" / "derivatives")
    assert rc == 0, err


def _reference_app_dirs():
    if not REF_APPS.is_dir():
        return []
    return sorted(p.parent for p in REF_APPS.rglob("main.cc"))


@needs_gxx
@needs_ref
def test_reference_apps_host_syntax():
    dirs = _reference_app_dirs()
    assert len(dirs) >= 10
    failed = {}
    for d in dirs:
        rc, err = host_syntax(d)
        if rc:
            failed[str(d.relative_to(REF_APPS))] = err[:400]
    assert not failed, failed


@pytest.mark.skipif(NVCC is None, reason="nvcc not available")
@needs_ref
@pytest.mark.parametrize("app,ok", [("allen_cahn/explicit", True), ("mechanics/eshelby_inclusion", True),
                                    ("cahn_hilliard/implicit", True), ("nucleation", False)])
def test_reference_apps_device_compile(tmp_path, app, ok):
    """The cell kernel compiles for the reference's own CustomPDE. An operator whose GPU callback
    calls a host-only function (nucleation's seed_nucleus) is rejected at compile time."""
    from phasefield_gb300 import app_build
    if ok:
        app_build.compile_app(REF_APPS / app, tmp_path / "main.o", link=False)
    else:
        with pytest.raises(RuntimeError, match="calling a __host__ function"):
            app_build.compile_app(REF_APPS / app, tmp_path / "main.o", link=False)


@pytest.mark.skipif(NVCC is None, reason="nvcc not available")
def test_example_app_device_compile_has_no_spills(tmp_path):
    from phasefield_gb300 import app_build
    d = EXAMPLES / "cahn_hilliard_explicit"
    r = subprocess.run([NVCC, *app_build.APP_FLAGS, "-Xptxas", "-v", "-I", str(INCLUDE), "-I", str(d), "-c",
                        str(d / "main.cc"), "-o", str(tmp_path / "m.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stderr.splitlines() if "spill stores" in l]
    assert lines and all("0 bytes spill stores, 0 bytes spill loads" in l for l in lines), lines


# ---------------------------------------------------------------------------------------------
# parameter files
# ---------------------------------------------------------------------------------------------
@needs_ref
def test_reference_parameter_files_parse(prm_dump):
    files = sorted(REF_APPS.rglob("*.prm"))
    assert len(files) >= 10
    for f in files:
        d = prm_dump(3, path=f)
        assert "error" not in d, (f, d)


def test_mesh_time_and_aliases(prm_dump):
    d = prm_dump(2, """
set global refinement = 3
subsection Rectangular mesh
  set x size = 10
  set y upper bound = 20   # alias of "y size"
  set x lower bound = 2
  set y subdivisions = 3
  set x periodic = true
end
set dt = 0.5
set number steps = 7
""")
    assert d["size"] == [10.0, 20.0] and d["lower"] == [2.0, 0.0] and d["subdivisions"] == [1, 3]
    assert d["periodic"] == [0] and d["refinement"] == 3
    assert d["dt"] == 0.5 and d["n_increments"] == 7
    # "end time" overrides the increment count: ceil((t_f - t_0) / dt)
    d = prm_dump(2, "set time step = 0.3\nset number steps = 5\nset end time = 1.0\n")
    assert d["n_increments"] == 4


def test_output_schedules(prm_dump):
    d = prm_dump(2, "set time step = 1\nset number steps = 100\nsubsection output\n set number = 4\nend\n")
    assert d["outputs"] == [0, 25, 50, 75, 100]
    d = prm_dump(2, "set time step = 1\nset number steps = 1000\nsubsection output\n set condition = LOG_SPACING\n"
                    " set number = 3\nend\n")
    assert d["outputs"] == [0, 10, 100, 1000]  # the default list adds increment 0
    d = prm_dump(2, "set time step = 1\nset number steps = 100\nsubsection output\n set condition = N_PER_DECADE\n"
                    " set number = 2\n set list = 33, 77\nend\n")
    assert d["outputs"] == [0, 1, 5, 10, 33, 50, 77, 100]


def test_boundary_conditions_and_linear_parameters(prm_dump):
    d = prm_dump(3, """
subsection boundary conditions: 0
  set variables = u:y, c
  set conditions = Dirichlet, Natural, Periodic, Periodic, Natural, Dirichlet
end
subsection linear solver parameters: 0
  set solver_ids = 1, 3
  set tolerance type = RMSEPerField
  set tolerance = 1e-8
  set preconditioner = GMG
  set mg_depth = 4
  subsection Chebyshev
    set smoother degree = 3
    set smoothing range = 20
  end
end
""")
    assert d["bcs"]["u"] == {"1": [1, 0, 3, 3, 0, 1]}
    assert d["bcs"]["c"] == {"0": [1, 0, 3, 3, 0, 1], "1": [1, 0, 3, 3, 0, 1], "2": [1, 0, 3, 3, 0, 1]}
    for sid in ("1", "3"):
        L = d["linear"][sid]
        assert (L["tolerance_type"], L["tolerance"], L["preconditioner"], L["mg_depth"]) == (1, 1e-8, 2, 4)
        assert (L["smoother_degree"], L["smoothing_range"], L["eig_cg_iterations"], L["max_iterations"]) == (3, 20, 10,
                                                                                                            100)


def test_model_constants(prm_dump):
    d = prm_dump(3, """
set Model constant a = 1.5, DOUBLE
set Model constant n = 4, INT
set Model constant flag = true, BOOL
set Model constant s = hello, STRING
set Model constant v = (1, 2, 3), TENSOR
set Model constant M = ((1,2,3),(4,5,6),(7,8,9)), TENSOR
set Model constant iso = (22.5, 0.3), isotropic elastic constants
set Model constant ortho = (10, 20, 30, 0.1, 0.2, 0.3, 4, 5, 6), orthotropic elastic constants
""")
    c = d["constants"]
    assert c["a"] == 1.5 and c["n"] == {"int": 4} and c["flag"] is True and c["s"] == "hello"
    assert c["v"] == [1, 2, 3] and c["M"] == [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
    E, nu = 22.5, 0.3
    lam, mu = nu * E / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    C = c["iso"]["voigt"]
    assert C[0][0] == pytest.approx(lam + 2 * mu, rel=1e-15) and C[0][1] == pytest.approx(lam, rel=1e-15)
    assert C[5][5] == pytest.approx(mu, rel=1e-15) and C[0][3] == 0.0
    # orthotropic: the compliance matrix inverted
    import numpy as np
    E1, E2, E3, n12, n13, n23, G12, G13, G23 = 10, 20, 30, 0.1, 0.2, 0.3, 4, 5, 6
    S = np.zeros((6, 6))
    S[0, 0], S[1, 1], S[2, 2] = 1 / E1, 1 / E2, 1 / E3
    S[0, 1] = S[1, 0] = -n12 / E1
    S[0, 2] = S[2, 0] = -n13 / E1
    S[1, 2] = S[2, 1] = -n23 / E2
    S[3, 3], S[4, 4], S[5, 5] = 1 / G23, 1 / G13, 1 / G12
    assert np.allclose(np.array(c["ortho"]["voigt"]), np.linalg.inv(S), rtol=1e-12, atol=1e-12)
    # 2-D plane stress isotropic
    d2 = prm_dump(2, "set Model constant iso = (22.5, 0.3), isotropic elastic constants planestress\n")
    C2 = d2["constants"]["iso"]["voigt"]
    assert C2[0][1] == pytest.approx(nu * E / (1 - nu * nu), rel=1e-15) and C2[2][2] == pytest.approx(mu, rel=1e-15)


def test_parameter_errors(prm_dump):
    assert "unknown parameter" in prm_dump(2, "set no such entry = 1\n")["error"]
    assert "Invalid boundary condition" in prm_dump(2, "subsection boundary conditions: 0\n set variables = c\n"
                                                       " set conditions = Dirichlet, Robin\nend\n")["error"]
    assert "error" in prm_dump(2, "subsection output\n set number = 3\n")  # unclosed subsection
    assert "error" in prm_dump(2, "set Model constant x = (1, 2), TENSOR\n")  # rank-1 needs 3 entries


def test_random_seed(prm_dump):
    d = prm_dump(2, "subsection miscellaneous\n set random seed = 7\nend\n")
    assert d["seed"] == 7
    assert prm_dump(2, "")["seed"] == 2025  # default seed of the reference


# ---------------------------------------------------------------------------------------------
# dependency sets: C++ header and the Python mirror agree
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("strings", [
    ["old_1(n)", "grad(old_1(n))"],
    ["n", "grad(n)", "hess(mu)", "lap(mu)", "src(n)", "grad(change(mu))", "old_4(mu)", "hessdiag(old_2(n))"],
    ["div(n)", "symgrad(lhs(mu))", "curl(trial(n))"],
])
def test_dependency_sets_match_python(prm_dump, strings):
    from phasefield_gb300.problem import FieldAttributes, make_dependency_set
    out = subprocess.run([str(prm_dump.exe), "--deps", "n,mu", *strings], capture_output=True, text=True,
                         check=True).stdout
    cpp = json.loads(out)
    py = make_dependency_set([FieldAttributes("n"), FieldAttributes("mu")], set(strings))
    assert set(cpp) == {str(k) for k in py}
    for k, d in py.items():
        flag, src, old = cpp[str(k)]
        assert (flag, src) == (d.flag, d.src_flag)
        assert old == list(d.old_flags)


def test_dependency_set_rejects_unknown(prm_dump):
    out = subprocess.run([str(prm_dump.exe), "--deps", "n", "grad(m)"], capture_output=True, text=True).stdout
    assert "not recognized" in json.loads(out)["error"]
