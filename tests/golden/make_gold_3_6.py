"""Extracts the reference's own recorded output of its Allen-Cahn regression run into
``prismspf_3_6_gold.json`` (run from the repository root, where the reference tree exists):

  python tests/golden/make_gold_3_6.py [reference root]

Source files (reference tree, read only here, never at test time):
  tests/regression_tests/prismspf_3_6/gold_output.txt   the log of a reference run: the DoF
      count (:9) and, at iterations 0, 300, ..., 1500, the l2-norm and integrated value of the
      three fields n, mg_n, f_tot (:28-60); 1500 explicit-solver calls (:69)
  tests/regression_tests/prismspf_3_6/custom_pde.h      the run's initial condition: twelve
      circular grains given by centre (fractions of 100) and radius, tanh profile width 1.5

The JSON holds those numbers as the reference printed them (six significant digits) plus the
configuration of the run that the log describes: 2-D, degree 1 (3 x 129^2 = 49,923 DoFs, i.e.
128^2 cells of [0,50]^2 at global refinement 7, uniform: the log says "grid refinement
disabled"), time step 0.01 for 1500 increments with 5 equally spaced outputs. The committed
parameters.prm beside the log is today's version of the test (degree 2 in main.cc, mesh
adaptivity on, time step 1e-3 to end time 15) and does not describe the logged run.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "prismspf_3_6_gold.json"


def main(ref_root: str = "/root/reference") -> None:
    d = Path(ref_root) / "tests" / "regression_tests" / "prismspf_3_6"
    log = (d / "gold_output.txt").read_text()
    pde = (d / "custom_pde.h").read_text()

    ndofs = int(re.search(r"number of degrees of freedom:\s*(\d+)", log).group(1))
    iterations = []
    for block in re.split(r"\n(?=Iteration: )", log)[1:]:
        it = int(re.match(r"Iteration: (\d+)", block).group(1))
        fields = {}
        for m in re.finditer(r"Solution index (\d+) l2-norm: (\S+) integrated value: (\S+)", block):
            fields[int(m.group(1))] = {"l2_norm": m.group(2), "integrated": m.group(3)}
        iterations.append({"iteration": it, "fields": [fields[i] for i in sorted(fields)]})
    n_explicit = int(re.search(r"\| Explicit solver\s*\|\s*(\d+)", log).group(1))

    table = re.search(r"center\[12\]\[3\]\s*=\s*\{(.*?)\};", pde, re.S).group(1)
    centres = [[float(x) for x in re.findall(r"[-\d.]+", row)] for row in re.findall(r"\{([^{}]*)\}", table)]
    radii = [float(x) for x in re.search(r"rad\[12\]\s*=\s*\{([^}]*)\}", pde).group(1).split(",")]
    width = float(re.search(r"std::tanh\(\(dist - rad\[i\]\) / ([\d.]+)\)", pde).group(1))
    scale = float(re.search(r"center\[i\]\[dir\] \* ([\d.]+)\)", pde).group(1))

    out = {
        "source": "tests/regression_tests/prismspf_3_6/gold_output.txt, custom_pde.h",
        "n_dofs_total": ndofs,
        "n_explicit_increments": n_explicit,
        "iterations": iterations,
        "field_names": ["n", "mg_n", "f_tot"],
        "initial_condition": {"centres": [[c[0] * scale, c[1] * scale] for c in centres], "radii": radii,
                              "width": width},
        "run": {"dim": 2, "degree": 1, "size": 50.0, "global_refinement": 7, "dt": 0.01,
                "n_increments": n_explicit, "output_every": n_explicit // 5, "m_well": 1.0, "kappa": 2.0},
    }
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main(*sys.argv[1:])
