"""The CUDA path against the reference's own recorded output: the log of its Allen-Cahn
regression run (tests/regression_tests/prismspf_3_6/gold_output.txt of the reference,
extracted to tests/golden/prismspf_3_6_gold.json).

* The engine, driven through the C ABI like the other parity tests, runs the logged
  configuration (Q1, 128^2 cells of [0,50]^2, twelve-grain initial condition, dt 0.01, 1500
  increments, post-processing on the 5 output increments); the l2-norm and integrated value of
  n, mg_n and f_tot must print as the reference printed them (six digits) at iterations 0, 300,
  ..., 1500.
* The drop-in C++ layer runs the same configuration as an application (tests/dropin/gold_3_6:
  main.cc, custom_pde.h and a parameter file): the log lines of its Problem::solve must carry
  the reference's numbers, and its interpolated initial condition (increment-0 output) must
  equal an independent evaluation of the initial condition at every support point (nodal
  interpolation, solver_base.h:178-229).
"""
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))

import gold_3_6 as G  # noqa: E402
from phasefield_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_engine_reproduces_reference_log(gpu_lib):
    wl = G.workload()
    p = wl.make_problem()
    jxw = 1.0 / p.invm()
    every = G.GOLD["run"]["output_every"]

    def norms(age):
        out = []
        for f in range(3):
            v = p.download(f, age=age) if f == 0 else p.download(f)
            out.append((float(np.linalg.norm(v)), float(v @ jxw)))
        return out

    p.solve(0, 1)  # increment 0: the post-processed fields of the initial condition
    bad = G.mismatches(0, norms(0))
    for it in range(every, G.GOLD["run"]["n_increments"] + 1, every):
        p.solve(it, every)
        bad += G.mismatches(it, norms(1))
    assert not bad, bad


def _write_ic_header(path: Path):
    ic = G.GOLD["initial_condition"]
    lines = ["#pragma once", f"#define GOLD_N {len(ic['radii'])}", f"#define GOLD_WIDTH {ic['width']!r}",
             "static const double gold_centres[GOLD_N][2] = {" +
             ", ".join("{%r, %r}" % (c[0], c[1]) for c in ic["centres"]) + "};",
             "static const double gold_radii[GOLD_N] = {" + ", ".join(repr(r) for r in ic["radii"]) + "};"]
    path.write_text("\n".join(lines) + "\n")


def test_dropin_application_reproduces_reference_log(gpu_lib, tmp_path):
    from phasefield_gb300 import app_build
    from test_gpu_dropin import read_vtu, to_lattice
    _write_ic_header(tmp_path / "gold_ic.h")
    exe = app_build.compile_app(ROOT / "tests" / "dropin" / "gold_3_6", tmp_path / "gold_3_6",
                                extra_flags=["-I" + str(tmp_path)])
    run = G.GOLD["run"]
    (tmp_path / "parameters.prm").write_text(f"""
subsection Rectangular mesh
  set x size = {run['size']}
  set y size = {run['size']}
  set x subdivisions = 1
  set y subdivisions = 1
end
set global refinement = {run['global_refinement']}
set time step = {run['dt']}
set end time = {run['dt'] * run['n_increments']}
subsection output
  set condition = EQUAL_SPACING
  set number = 5
end
""")
    r = subprocess.run([str(exe), "-i", "parameters.prm"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    printed = {}
    for block in r.stdout.split("Iteration ")[1:]:
        it = int(block.split()[0])
        printed[it] = [(m.group(1), m.group(2)) for m in
                       re.finditer(r"Field index \d+ name \S+ l2-norm (\S+) integrated value (\S+)", block)]
    assert sorted(printed) == [rec["iteration"] for rec in G.GOLD["iterations"]]
    bad = []
    for rec in G.GOLD["iterations"]:
        got = printed[rec["iteration"]]
        bad += G.mismatches(rec["iteration"], [(float(a), float(b)) for a, b in got])
        for (a, b), ref in zip(got, rec["fields"]):  # the printed strings themselves
            if (a, b) != (ref["l2_norm"], ref["integrated"]):
                bad.append((rec["iteration"], a, b, ref))
    assert not bad, bad

    # nodal interpolation of the initial condition at every support point
    wl = G.workload()
    digits = len(str(run["n_increments"]))  # output files are numbered with the last increment's width
    v0 = read_vtu(tmp_path / "solutions" / ("solution_" + "0" * digits + ".vtu"))
    n0 = to_lattice(v0, wl.mesh, "n")
    ref = G.initial_condition(W.lattice_coordinates(wl.mesh))
    assert np.max(np.abs(n0 - ref)) <= 1e-15  # host libm tanh/sqrt against numpy's: a few ulps
