"""GPU test of the allocation-free Allen-Cahn step (ppf_allen_cahn_step_noalloc).

That entry point serves callers that cannot allocate GPU memory at the point where they need
a step (a host framework that owns every device allocation through its own pool, or a
fixed-memory loop where cudaMalloc/cudaFree are not allowed): it takes caller-owned input
and output vectors and keeps its scratch in a static device array. This test calls it
through the C ABI twice in a row (the second call on the first call's output, so stale
scratch from the first call would show) and compares each result with the handle-based
explicit solve of the same block, at the 1e-12 relative L2 bar of one operator apply, for
degrees 1 to 4 (the tables of degrees 3 and 4 are built by the entry point's own closed-form
Gauss-Lobatto rules). The companion status call reports a clean step as PPF_OK and a step on
an input holding a NaN as PPF_ERR_NAN.

The file is named to be collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from phasefield_gb300 import capi
from phasefield_gb300 import workloads as W
from phasefield_gb300.problem import RectangularMesh

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def allen_cahn(dim, degree, refine):
    wl = W.allen_cahn_2d(refine=refine, degree=degree, dt=0.01)
    if dim == 3:
        wl.mesh = RectangularMesh(dim=3, degree=degree, size=(100.0, 100.0, 100.0), global_refinement=refine)
        x = W.lattice_coordinates(wl.mesh)
        rng = np.random.default_rng(21)
        wl.initial = {0: W.grain_field(x, rng.uniform(0, 100, (12, 3)), rng.uniform(10, 25, 12), 2.0)}
    return wl


def mesh_desc(mesh):
    m = capi.MeshDesc()
    m.dim, m.degree, m.global_refinement = mesh.dim, mesh.degree, mesh.global_refinement
    for d in range(3):
        m.subdivisions[d] = mesh.subdivisions[d] if d < mesh.dim else 1
        m.lower[d] = mesh.lower[d] if d < mesh.dim else 0.0
        m.size[d] = mesh.size[d] if d < mesh.dim else 1.0
        m.periodic[d] = 0
    return m


@pytest.mark.parametrize("dim,degree,refine", [(2, 1, 5), (2, 2, 4), (2, 3, 3), (3, 2, 2), (3, 4, 1)])
def test_noalloc_step_matches_handle_step_twice(gpu_lib, dim, degree, refine):
    import torch

    wl = allen_cahn(dim, degree, refine)
    m_well, kappa = wl.constants
    # existing entry points: two explicit solves of block 1 through a handle
    p = wl.make_problem()
    n0 = wl.initial[0]
    p.upload(0, n0, age=1)
    p.solve_block(0)
    ref1 = p.download(0, age=0)
    p.upload(0, ref1, age=1)
    p.solve_block(0)
    ref2 = p.download(0, age=0)
    p.close()

    # the allocation-free entry point on caller-owned device vectors, twice in a row
    lib = capi.load()
    m = mesh_desc(wl.mesh)
    d_in = torch.from_numpy(np.ascontiguousarray(n0)).cuda()
    d_out1 = torch.full_like(d_in, float("nan"))
    d_out2 = torch.full_like(d_in, float("nan"))
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), m_well, kappa, wl.dt, C.c_void_p(d_in.data_ptr()),
                                         C.c_void_p(d_out1.data_ptr()), stream)
    assert rc == capi.PPF_OK
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), m_well, kappa, wl.dt, C.c_void_p(d_out1.data_ptr()),
                                         C.c_void_p(d_out2.data_ptr()), stream)
    assert rc == capi.PPF_OK
    assert lib.ppf_allen_cahn_step_noalloc_status(stream) == capi.PPF_OK
    torch.cuda.synchronize()
    out1, out2 = d_out1.cpu().numpy(), d_out2.cpu().numpy()
    assert rel_l2(out1, ref1) < TOL
    assert rel_l2(out2, ref2) < TOL


def test_noalloc_status_reports_a_nonfinite_step(gpu_lib):
    import torch

    wl = allen_cahn(2, 1, 4)
    m_well, kappa = wl.constants
    lib = capi.load()
    m = mesh_desc(wl.mesh)
    n0 = wl.initial[0].copy()
    n0[37] = np.nan  # planted on the host
    d_in = torch.from_numpy(n0).cuda()
    d_out = torch.empty_like(d_in)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), m_well, kappa, wl.dt, C.c_void_p(d_in.data_ptr()),
                                         C.c_void_p(d_out.data_ptr()), stream)
    assert rc == capi.PPF_OK
    assert lib.ppf_allen_cahn_step_noalloc_status(stream) == capi.PPF_ERR_NAN
    # the next step clears the word
    d_in = torch.from_numpy(wl.initial[0].copy()).cuda()
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), m_well, kappa, wl.dt, C.c_void_p(d_in.data_ptr()),
                                         C.c_void_p(d_out.data_ptr()), stream)
    assert rc == capi.PPF_OK
    assert lib.ppf_allen_cahn_step_noalloc_status(stream) == capi.PPF_OK


def test_noalloc_rejects_meshes_above_the_limit(gpu_lib):
    import torch

    lib = capi.load()
    # 1025 x 1025 lattice nodes (Q1, 1024^2 cells) exceeds the 1,048,576-node limit
    mesh = RectangularMesh(dim=2, degree=1, size=(1.0, 1.0), global_refinement=10)
    m = mesh_desc(mesh)
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), 1.0, 1.0, 0.01, C.c_void_p(d.data_ptr()),
                                         C.c_void_p(d.data_ptr()), None)
    assert rc == capi.PPF_ERR_UNSUPPORTED
    # a refinement whose cell count overflows 32 bits is rejected, not wrapped to a small mesh
    m.global_refinement = 31
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), 1.0, 1.0, 0.01, C.c_void_p(d.data_ptr()),
                                         C.c_void_p(d.data_ptr()), None)
    assert rc == capi.PPF_ERR_ARG
    m.global_refinement, m.subdivisions[0] = 24, 1 << 8
    rc = lib.ppf_allen_cahn_step_noalloc(C.byref(m), 1.0, 1.0, 0.01, C.c_void_p(d.data_ptr()),
                                         C.c_void_p(d.data_ptr()), None)
    assert rc == capi.PPF_ERR_UNSUPPORTED
