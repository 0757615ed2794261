"""The oracle against the one record of its own output that the reference ships: the log of
its Allen-Cahn regression run (tests/regression_tests/prismspf_3_6/gold_output.txt, extracted
to tests/golden/prismspf_3_6_gold.json).

The oracle runs the logged configuration (Q1, 128^2 cells of [0,50]^2, the test's twelve-grain
initial condition, dt 0.01, 1500 increments, post-processing on the 5 output increments) and
every number the reference printed must come out the same to the printed six digits: the DoF
count, and the l2-norm (``Vector::l2_norm``) and integrated value (the vector dotted with the
lumped JxW, problem.cc:517-548) of n, mg_n and f_tot at iterations 0, 300, ..., 1500.
"""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))

import gold_3_6 as G  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def test_fixture_describes_the_logged_run():
    run = G.GOLD["run"]
    n1 = run["degree"] * 2 ** run["global_refinement"] + 1
    assert G.GOLD["n_dofs_total"] == 3 * n1 * n1
    assert [r["iteration"] for r in G.GOLD["iterations"]] == list(range(0, 1501, 300))
    assert G.GOLD["n_explicit_increments"] == run["n_increments"] == 1500


def test_matches_printed_rounding():
    assert G.matches_printed(109.4584999, "109.458")
    assert not G.matches_printed(109.4586, "109.458")
    assert G.matches_printed(8.07180, "8.0718")
    assert not G.matches_printed(8.07186, "8.0718")


def test_oracle_reproduces_reference_log():
    wl = G.workload()
    o = po.Oracle(wl)
    assert 3 * o.n_dofs(0) == G.GOLD["n_dofs_total"]  # three scalar fields
    jxw = 1.0 / o.invm(0)

    def norms(current_age):
        out = []
        for f in range(3):
            v = o.get(f, current_age if f == 0 else 0)
            out.append((float(np.linalg.norm(v)), float(v @ jxw)))
        return out

    assert o.run(0, 1) == 0  # increment 0: initial condition and the post-processed fields
    bad = G.mismatches(0, norms(0))
    every = G.GOLD["run"]["output_every"]
    for it in range(every, G.GOLD["run"]["n_increments"] + 1, every):
        assert o.run(it, every) == 0
        bad += G.mismatches(it, norms(1))  # after the increment's rotation n is old_1
    assert not bad, bad
