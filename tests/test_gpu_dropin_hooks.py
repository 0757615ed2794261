"""The drop-in's solve-block hooks and user stop on the GPU (reference: PDEOperatorBase::
pre_solve_block / post_solve_block / set_user_stop, include/prismspf/core/pde_operator_base.h:
96-138, called by Problem::solve_increment, src/core/problem.cc:436-477, with exit status 3 and
forced output, :392-414).

The application tests/dropin/hooks overrides both hooks: they print every call with the
increment and time of the SolveContext's timer, the post hook of block 1 prints the sum of n
read through the context, and at increment 7 it calls set_user_stop(true). Checked: the hooks
run exactly around the blocks that are solved (block 1 every increment, the post-processing
block 2 on output increments 0 and 5 only), the run stops after increment 7 with its output
written and the reference's message, and the sums and the final field match the oracle
(1e-12 relative for the sums, 1e-9 relative L2 for the field).
"""
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))

import gold_3_6 as G  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from phasefield_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
STOP, N, REFINE, DT = 7, 20, 5, 0.01


def test_hooks_and_user_stop(gpu_lib, tmp_path):
    from phasefield_gb300 import app_build
    from test_gpu_dropin import read_vtu, to_lattice
    from test_gpu_gold_3_6 import _write_ic_header
    _write_ic_header(tmp_path / "gold_ic.h")
    exe = app_build.compile_app(ROOT / "tests" / "dropin" / "hooks", tmp_path / "hooks",
                                extra_flags=["-I" + str(tmp_path)])
    (tmp_path / "parameters.prm").write_text(f"""
subsection Rectangular mesh
  set x size = 50
  set y size = 50
end
set global refinement = {REFINE}
set time step = {DT}
set number steps = {N}
subsection output
  set condition = EQUAL_SPACING
  set number = 4
end
set Model constant stop_increment = {STOP}, INT
""")
    r = subprocess.run([str(exe), "-i", "parameters.prm"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    calls = [(m.group(1), int(m.group(2)), int(m.group(3)), float(m.group(4)))
             for m in re.finditer(r"hook (pre|post) (\d+) (\d+) (\S+)", r.stdout)]
    expected = []
    for inc in range(STOP + 1):
        blocks = [1, 2] if inc in (0, 5) else [1]
        for b in blocks:
            expected += [("pre", b, inc), ("post", b, inc)]
    assert [c[:3] for c in calls] == expected
    assert all(abs(t - inc * DT) < 1e-12 for _, _, inc, t in calls)
    assert "Exit triggered by user!" in r.stdout
    files = sorted(p.name for p in (tmp_path / "solutions").glob("solution_*.vtu"))
    assert files == ["solution_00.vtu", "solution_05.vtu", f"solution_{STOP:02d}.vtu"]

    wl = W.allen_cahn_2d(refine=REFINE, degree=1, size=50.0, dt=DT)
    wl.initial = {0: G.initial_condition(W.lattice_coordinates(wl.mesh))}
    o = po.Oracle(wl)
    sums = {int(m.group(1)): float(m.group(2)) for m in re.finditer(r"hook sum (\d+) (\S+)", r.stdout)}
    assert sorted(sums) == list(range(STOP + 1))
    for inc in range(STOP + 1):
        assert o.run(inc, 5) == 0
        ref = o.get(0, 1)  # after the increment's rotation
        assert abs(sums[inc] - ref.sum()) <= 1e-12 * abs(ref.sum()), inc
    got = to_lattice(read_vtu(tmp_path / "solutions" / f"solution_{STOP:02d}.vtu"), wl.mesh, "n")
    assert np.linalg.norm(got - ref) <= 1e-9 * np.linalg.norm(ref)
