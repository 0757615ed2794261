"""Batched ensembles of independent explicit Allen-Cahn simulations over the C ABI.

``Ensemble`` wraps ppf_ensemble_*: instances of uneven mesh size (2-D, natural boundaries),
degree 1 or 2 and parameters (m_well, kappa), advanced by one kernel launch per step.
``allen_cahn_ensemble`` builds the seeded 256-instance workload: cells per side drawn from
32..256 (subdivisions x 2^r), degree 1 or 2, m_well in [0.5, 2], kappa in [1, 4], grain
initial conditions (12 grains, radius 5-15, tanh width 2) on [0,100]^2.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .problem import RectangularMesh
from .workloads import grain_field, lattice_coordinates


def _bind(lib):
    if getattr(lib, "_ens_bound", False):
        return lib
    P = C.POINTER
    dp = P(C.c_double)
    E = C.c_void_p
    lib.ppf_ensemble_create.argtypes = [C.c_int, P(capi.MeshDesc), dp, dp, C.c_double, P(E)]
    lib.ppf_ensemble_destroy.argtypes = [E]
    lib.ppf_ensemble_destroy.restype = None
    lib.ppf_ensemble_last_error.argtypes = [E]
    lib.ppf_ensemble_last_error.restype = C.c_char_p
    lib.ppf_ensemble_instance_length.argtypes = [E, C.c_int]
    lib.ppf_ensemble_instance_length.restype = C.c_longlong
    lib.ppf_ensemble_upload.argtypes = [E, C.c_int, dp]
    lib.ppf_ensemble_download.argtypes = [E, C.c_int, dp]
    lib.ppf_ensemble_run.argtypes = [E, C.c_int, C.c_int]
    lib.ppf_ensemble_autotune.argtypes = [E, C.c_int, dp, P(C.c_int), P(C.c_int)]
    lib.ppf_ensemble_synchronize.argtypes = [E]
    lib.ppf_ensemble_set_stream.argtypes = [E, C.c_void_p]
    lib._ens_bound = True
    return lib


def mesh_desc(mesh: RectangularMesh) -> capi.MeshDesc:
    m = capi.MeshDesc()
    m.dim, m.degree, m.global_refinement = mesh.dim, mesh.degree, mesh.global_refinement
    for d in range(3):
        m.subdivisions[d] = mesh.subdivisions[d] if d < mesh.dim else 1
        m.lower[d] = mesh.lower[d] if d < mesh.dim else 0.0
        m.size[d] = mesh.size[d] if d < mesh.dim else 1.0
        m.periodic[d] = int(mesh.periodic[d]) if d < mesh.dim else 0
    return m


class Ensemble:
    def __init__(self, meshes: list[RectangularMesh], m_well, kappa, dt: float):
        self.lib = _bind(capi.load())
        self.meshes = meshes
        n = len(meshes)
        md = (capi.MeshDesc * n)(*[mesh_desc(m) for m in meshes])
        mw = np.ascontiguousarray(m_well, dtype=np.float64)
        ka = np.ascontiguousarray(kappa, dtype=np.float64)
        h = C.c_void_p()
        rc = self.lib.ppf_ensemble_create(n, md, capi.dptr(mw), capi.dptr(ka), float(dt), C.byref(h))
        if rc != capi.PPF_OK:
            raise capi.PPFError(rc, "ensemble creation failed")
        self.h = h

    def _check(self, rc):
        if rc != capi.PPF_OK:
            raise capi.PPFError(rc, self.lib.ppf_ensemble_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.ppf_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, i: int, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.lib.ppf_ensemble_upload(self.h, i, capi.dptr(v)))

    def download(self, i: int) -> np.ndarray:
        out = np.empty(int(self.lib.ppf_ensemble_instance_length(self.h, i)))
        self._check(self.lib.ppf_ensemble_download(self.h, i, capi.dptr(out)))
        return out

    def run(self, n_steps: int, use_graph: bool = True):
        self._check(self.lib.ppf_ensemble_run(self.h, n_steps, int(use_graph)))

    def autotune(self, steps: int = 5):
        ms, shape, grid = C.c_double(), C.c_int(), C.c_int()
        self._check(self.lib.ppf_ensemble_autotune(self.h, steps, C.byref(ms), C.byref(shape), C.byref(grid)))
        return ms.value, shape.value, grid.value

    def synchronize(self):
        self._check(self.lib.ppf_ensemble_synchronize(self.h))

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.ppf_ensemble_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None))


def allen_cahn_ensemble(n_instances: int = 256, seed: int = 2024, min_cells: int = 32, max_cells: int = 256,
                        size: float = 100.0):
    """Meshes, parameters and initial conditions of the seeded ensemble workload."""
    rng = np.random.default_rng(seed)
    meshes, mw, ka, ics = [], [], [], []
    for _ in range(n_instances):
        cells = int(rng.integers(min_cells, max_cells + 1))
        # cells = subdivisions x 2^r with the largest r that keeps subdivisions integral
        r = 0
        while cells % (2 ** (r + 1)) == 0 and r < 8:
            r += 1
        sub = cells // (2 ** r)
        degree = int(rng.integers(1, 3))
        mesh = RectangularMesh(dim=2, degree=degree, size=(size, size), subdivisions=(sub, sub, 1),
                               global_refinement=r)
        meshes.append(mesh)
        mw.append(float(rng.uniform(0.5, 2.0)))
        ka.append(float(rng.uniform(1.0, 4.0)))
        x = lattice_coordinates(mesh)
        centres = rng.uniform(0.0, size, size=(12, 2))
        radii = rng.uniform(5.0, 15.0, size=12)
        ics.append(grain_field(x, centres, radii, 2.0))
    return meshes, np.array(mw), np.array(ka), ics
