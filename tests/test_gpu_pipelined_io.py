"""Pipelined host I/O (ppf_upload_state_staged, ppf_run_async, ppf_wait) against the blocking
path (ppf_upload_state, ppf_run, ppf_download_solution).

Every increment takes its inputs from a host buffer and streams its results back, as a caller
that keeps its state on the host does. The queued form lets the next increment's uploads start
while the current one computes; the staging protocol must still hand every increment exactly
the inputs staged for it. Checked with two different input sets alternating between increments
(a staged upload that overtook the run consuming the previous one would swap them): the
streamed results equal the blocking path's within 1e-14 relative L2 (same kernels and
contraction mode; only the order of the atomic accumulation may differ), and a NaN staged for
one increment is reported by ppf_wait.
"""
import ctypes as C

import numpy as np
import pytest

from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _wl():
    return W.cahn_hilliard_3d(refine=3, degree=2, size=8.0, dt=1e-4)


def _ptr(t):
    return C.cast(t.data_ptr(), C.POINTER(C.c_double))


def _inputs(N):
    rng = np.random.default_rng(31)
    sets = []
    for _ in range(2):
        c = 0.5 + 0.05 * rng.uniform(-1, 1, N)
        mu = 0.1 * rng.uniform(-1, 1, N)
        sets.append((c, mu))
    return sets


def test_queued_increments_match_blocking_increments(gpu_lib, monkeypatch):
    import torch
    monkeypatch.setenv("PPF_CONTRACTION_MODE", "1")  # the same arithmetic in both handles
    n_steps = 6
    wl = _wl()
    ref = wl.make_problem()
    ref.solve(0)
    N = ref.n_nodes
    sets = _inputs(N)
    expected = []
    for k in range(n_steps):
        c, mu = sets[k % 2]
        ref.upload(0, c, age=1)
        ref.upload(1, mu, age=1)
        ref.solve(k + 1)
        expected.append((ref.download_solution(0), ref.download_solution(1)))

    p = wl.make_problem()
    p.solve(0)
    pin_in = [[torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for v in s] for s in sets]
    pin_out = [torch.empty(N, dtype=torch.float64, pin_memory=True) for _ in range(2)]
    for f in (0, 1):
        p.set_output_stream(f, pin_out[f])
    lib = p.lib
    got = []
    for k in range(n_steps):
        for f in (0, 1):
            assert lib.ppf_upload_state_staged(p.h, f, 1, _ptr(pin_in[k % 2][f])) == capi.PPF_OK
        assert lib.ppf_run_async(p.h, k + 1, 0) == capi.PPF_OK
        if k in (2, n_steps - 1):  # queued increments, then read back after a wait
            assert lib.ppf_wait(p.h) == capi.PPF_OK
            got.append((k, pin_out[0].numpy().copy(), pin_out[1].numpy().copy()))
    for k, c, mu in got:
        assert rel_l2(c, expected[k][0]) < 1e-14, k
        assert rel_l2(mu, expected[k][1]) < 1e-14, k
    # the state after the queued increments is the blocking path's
    assert rel_l2(p.download_solution(0), expected[-1][0]) < 1e-14


def test_wait_reports_a_nonfinite_increment(gpu_lib):
    import torch
    wl = _wl()
    p = wl.make_problem()
    p.solve(0)
    N = p.n_nodes
    c, mu = _inputs(N)[0]
    mu = mu.copy()
    mu[N // 3] = np.nan  # planted on the host
    pins = [torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for v in (c, mu)]
    for f in (0, 1):
        assert p.lib.ppf_upload_state_staged(p.h, f, 1, _ptr(pins[f])) == capi.PPF_OK
    assert p.lib.ppf_run_async(p.h, 1, 0) == capi.PPF_OK
    assert p.lib.ppf_wait(p.h) == capi.PPF_ERR_NAN


def test_staged_upload_before_graph_replays(gpu_lib, monkeypatch):
    """A staged upload swaps a new buffer into the state: an increment graph captured on the
    former buffers must not be replayed. Runs of several increments (graph replays from increment
    2 on) after staged uploads give the blocking path's fields."""
    monkeypatch.setenv("PPF_CONTRACTION_MODE", "1")
    wl = _wl()
    ref = wl.make_problem()
    p = wl.make_problem()
    for h in (ref, p):
        h.solve(0)
    N = ref.n_nodes
    sets = _inputs(N)
    import torch
    pin_in = [[torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for v in s] for s in sets]
    lib = p.lib
    inc = 0
    for r in range(3):
        c, mu = sets[r % 2]
        ref.upload(0, c, age=1)
        ref.upload(1, mu, age=1)
        for f in (0, 1):
            assert lib.ppf_upload_state_staged(p.h, f, 1, _ptr(pin_in[r % 2][f])) == capi.PPF_OK
        inc += 6
        ref.solve(inc)
        assert lib.ppf_run_async(p.h, inc, 0) == capi.PPF_OK
        assert lib.ppf_wait(p.h) == capi.PPF_OK
        # six increments of atomic-accumulation rounding (a graph replayed on the former
        # buffers would differ by O(1))
        for f in (0, 1):
            assert rel_l2(p.download_solution(f), ref.download_solution(f)) < 1e-12, (r, f)
