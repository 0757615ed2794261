"""Streamed outputs (ppf_set_output_stream): after every increment the host buffer holds what
ppf_download_solution returns — for explicitly solved fields (copied on a copy stream while the
later blocks compute) and for a field written by a linear solve (copied at the end of the
increment) — into pageable or pinned memory; streaming stops when the buffer is unset."""
import numpy as np
import pytest

from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pinned", [False, True])
def test_explicit_fields_stream_each_increment(gpu_lib, pinned):
    wl = W.cahn_hilliard_3d(refine=2, degree=2, dim=3, size=8.0, dt=1e-4)
    p = wl.make_problem()
    p.solve(0)
    n = p.field_length(0)
    if pinned:
        import torch
        bufs = [torch.zeros(n, dtype=torch.float64, pin_memory=True) for _ in range(2)]
        view = [b.numpy() for b in bufs]
    else:
        bufs = [np.zeros(n) for _ in range(2)]
        view = bufs
    for f in (0, 1):
        p.set_output_stream(f, bufs[f])
    for inc in (1, 2, 3):
        p.solve(inc)
        for f in (0, 1):
            assert np.array_equal(view[f], p.download_solution(f)), (inc, f)
    p.set_output_stream(1, None)
    before = view[1].copy()
    p.solve(4)
    assert np.array_equal(view[0], p.download_solution(0))
    assert np.array_equal(view[1], before)  # no longer streamed
    assert not np.array_equal(before, p.download_solution(1))


def test_linear_field_streams_at_the_end_of_the_increment(gpu_lib):
    wl = W.eshelby_3d(refine=1, degree=2, size=16.0, n_incl=3, dim=3)
    p = wl.make_problem()
    buf = np.zeros(p.field_length(0))
    p.set_output_stream(0, buf)
    p.solve(1)
    assert np.linalg.norm(buf) > 0
    assert np.array_equal(buf, p.download_solution(0))


def test_streamed_output_arguments(gpu_lib):
    wl = W.cahn_hilliard_3d(refine=1, degree=1, dim=3, size=4.0)
    p = wl.make_problem()
    with pytest.raises(ValueError):
        p.set_output_stream(0, np.zeros(3))
    buf = np.zeros(p.field_length(0))
    rc = p.lib.ppf_set_output_stream(p.h, 0, capi.dptr(buf), capi.ORDER_DEALII)
    assert rc == capi.PPF_ERR_UNSUPPORTED
    assert p.lib.ppf_set_output_stream(p.h, 7, None, capi.ORDER_LATTICE) == capi.PPF_ERR_ARG


def test_async_upload_is_read_by_the_next_solve(gpu_lib):
    """ppf_upload_state_async queues the copy on the handle's stream: the increment after it
    sees the uploaded state as after ppf_upload_state."""
    import torch
    outs = []
    for use_async in (False, True):
        wl = W.cahn_hilliard_3d(refine=2, degree=2, dim=3, size=8.0, dt=1e-4)
        p = wl.make_problem()
        p.solve(0)
        rng = np.random.default_rng(4)
        host = torch.from_numpy(0.5 + 0.05 * rng.uniform(-1, 1, p.field_length(0))).pin_memory()
        ptr = capi.dptr(host.numpy())
        if use_async:
            assert p.lib.ppf_upload_state_async(p.h, 0, 1, ptr, capi.ORDER_LATTICE) == 0
        else:
            assert p.lib.ppf_upload_state(p.h, 0, 1, ptr, capi.ORDER_LATTICE) == 0
        p.solve(1)
        outs.append(p.download_solution(0))
    # the scatter's FP64 atomics may add in another order from run to run
    assert np.linalg.norm(outs[0] - outs[1]) <= 1e-13 * np.linalg.norm(outs[0])
