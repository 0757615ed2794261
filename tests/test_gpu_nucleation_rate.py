"""NucleationRate solve blocks on the GPU against the oracle.

The reference solves a NucleationRate block on output increments and on nucleation-attempt
increments, i.e. increments divisible by the `nucleation period` (problem.cc:436-443,
nucleation_parameters.cc:110-113), and skips it otherwise. The Allen-Cahn workload's second
block (|grad n| and the free-energy density) is declared NucleationRate here; with outputs
every 10 increments and a nucleation period of 7 it must run at increments 0, 7, 10, 14, 20,
21, 28, 30 and keep its fields in between. Bars: fields within 1e-9 relative L2 of the
oracle after every increment (plain launches), and the CUDA-graph replay of the increment
loop, which must stop at every due increment, gives the plain result within 1e-12.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import workloads as W
from phasefield_gb300.problem import NucleationRate

pytestmark = pytest.mark.gpu

TOL = 1e-9
PERIOD, OUTPUT_EVERY, LAST = 7, 10, 30


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def workload():
    wl = W.allen_cahn_2d(refine=4, degree=2, dt=0.01)
    wl.blocks[1].solve_timing = NucleationRate
    return wl


def test_nucleation_rate_block_runs_on_its_increments(gpu_lib):
    wl = workload()
    p = wl.make_problem()
    p.lib.ppf_set_use_graph(p.h, 0)
    p.set_nucleation_period(PERIOD)
    o = po.Oracle(wl)
    o.set_nucleation_period(PERIOD)
    due = {k for k in range(LAST + 1) if k % PERIOD == 0 or k % OUTPUT_EVERY == 0}
    prev = None
    for k in range(LAST + 1):
        p.solve(k, OUTPUT_EVERY)
        assert o.run(k, OUTPUT_EVERY) == 0
        mg = p.download(1)
        assert rel_l2(mg, o.get(1, 0)) < TOL, k
        assert rel_l2(p.download(2), o.get(2, 0)) < TOL, k
        assert rel_l2(p.download(0, age=1), o.get(0, 1)) < TOL, k
        if prev is not None:
            # the block's fields change exactly on the increments where it is due
            assert (not np.array_equal(mg, prev)) == (k in due), k
        prev = mg


def test_graph_replay_stops_at_nucleation_increments(gpu_lib):
    res = []
    for use_graph in (0, 1):
        p = workload().make_problem()
        p.lib.ppf_set_use_graph(p.h, use_graph)
        p.set_nucleation_period(PERIOD)
        p.solve(LAST + 3)  # no outputs: the block runs at 0, 7, 14, 21, 28 only
        res.append([p.download(f, age=1 if f == 0 else 0) for f in (0, 1, 2)])
        p.close()
    o = po.Oracle(workload())
    o.set_nucleation_period(PERIOD)
    assert o.run(LAST + 3) == 0
    for f in (0, 1, 2):
        assert rel_l2(res[1][f], res[0][f]) < 1e-12, f
        assert rel_l2(res[0][f], o.get(f, 1 if f == 0 else 0)) < TOL, f
