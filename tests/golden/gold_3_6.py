"""Helpers for the reference's recorded Allen-Cahn run (``prismspf_3_6_gold.json``, made by
``make_gold_3_6.py`` from the reference's tests/regression_tests/prismspf_3_6/gold_output.txt).

The reference printed its norms with an output stream's default six significant digits, so a
value reproduces the log when it lies within half a unit of the sixth digit of the printed
number (the printed string is what the comparison rests on).
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
GOLD = json.loads((HERE / "prismspf_3_6_gold.json").read_text())


def initial_condition(x: np.ndarray) -> np.ndarray:
    """The run's initial n at points x (shape (N, 2)): sum of the twelve grains' tanh profiles,
    capped at 1, as the regression test's set_initial_condition accumulates them."""
    ic = GOLD["initial_condition"]
    s = np.zeros(x.shape[0])
    for c, r in zip(ic["centres"], ic["radii"]):
        d = np.sqrt(((x - np.asarray(c)[None, :]) ** 2).sum(1))
        s += 0.5 * (1.0 - np.tanh((d - r) / ic["width"]))
    return np.minimum(s, 1.0)


def workload():
    """The logged run as a workload of this package: 2-D Allen-Cahn with the post-processed
    fields mg_n and f_tot, Q1, 128^2 cells of [0,50]^2, dt 0.01."""
    from phasefield_gb300 import workloads as W
    run = GOLD["run"]
    wl = W.allen_cahn_2d(refine=run["global_refinement"], degree=run["degree"], size=run["size"], dt=run["dt"],
                         m_well=run["m_well"], kappa=run["kappa"], n_steps=run["n_increments"])
    wl.initial = {0: initial_condition(W.lattice_coordinates(wl.mesh))}
    return wl


def matches_printed(value: float, printed: str) -> bool:
    """True when `value` printed with six significant digits gives `printed` (half a unit of
    the last printed digit, with a relative slack of 1e-9 for a value on a rounding tie)."""
    g = float(printed)
    if g == 0.0:
        return abs(value) < 5e-7
    unit = 10.0 ** (math.floor(math.log10(abs(g))) - 5)
    return abs(value - g) <= 0.5 * unit * (1.0 + 1e-9) + 1e-9 * abs(g)


def mismatches(iteration: int, values) -> list:
    """Compares [(l2_norm, integrated) per field] at one logged iteration; returns the misses."""
    rec = next(r for r in GOLD["iterations"] if r["iteration"] == iteration)
    bad = []
    for f, ((l2, integral), ref) in enumerate(zip(values, rec["fields"])):
        if not matches_printed(l2, ref["l2_norm"]):
            bad.append((iteration, f, "l2_norm", l2, ref["l2_norm"]))
        if not matches_printed(integral, ref["integrated"]):
            bad.append((iteration, f, "integrated", integral, ref["integrated"]))
    return bad
