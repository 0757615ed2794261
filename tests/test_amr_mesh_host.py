"""The engine's host-side adaptive mesh (phasefield_gb300/csrc/amr_mesh.cu: hash-based forest,
smoothing, numbering, hanging-node lines, transfer plan) against the oracle's brute-force
restatement, on the CPU: from the same random refine/coarsen marks both must reach the same
cells in the same order, the same DoF numbering and hanging lines, and the same transferred
fields. amr_mesh.cu is plain C++; the test compiles it with g++ and tests/amr_mesh_shim.cc."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po
from phasefield_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "phasefield_gb300" / "csrc"

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("amr_shim") / "libamr_shim.so"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-I", str(CSRC), "-x", "c++",
           str(CSRC / "amr_mesh.cu"), "-x", "c++", str(ROOT / "tests" / "amr_mesh_shim.cc"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(out))
    ip, dp, V = C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p
    lib.shim_uniform.restype = V
    lib.shim_uniform.argtypes = [C.c_int, C.c_int, ip, ip, C.c_int, C.c_int]
    lib.shim_free.argtypes = [V]
    for f in ("shim_ncells", "shim_ndofs"):
        getattr(lib, f).restype = C.c_longlong
        getattr(lib, f).argtypes = [V]
    lib.shim_cells.argtypes = [V, ip]
    lib.shim_cell_dofs.argtypes = [V, ip]
    lib.shim_hanging.restype = C.c_longlong
    lib.shim_hanging.argtypes = [V, ip, ip, dp]
    lib.shim_refine.restype = V
    lib.shim_refine.argtypes = [V, C.POINTER(C.c_byte), C.c_int]
    lib.shim_transfer.restype = C.c_longlong
    lib.shim_transfer.argtypes = [V, V, ip, ip, dp]
    return lib


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Mesh:
    def __init__(self, lib, ptr):
        self.lib, self.p = lib, ptr

    def cells(self):
        out = np.zeros((self.lib.shim_ncells(self.p), 4), np.int32)
        self.lib.shim_cells(self.p, _ip(out))
        return out

    def cell_dofs(self, nq):
        out = np.zeros(self.lib.shim_ncells(self.p) * nq, np.int32)
        self.lib.shim_cell_dofs(self.p, _ip(out))
        return out

    def hanging(self):
        n = self.lib.shim_ndofs(self.p)
        t = self.lib.shim_hanging(self.p, None, None, None)
        cnt, mas, w = np.zeros(n, np.int32), np.zeros(max(t, 1), np.int32), np.zeros(max(t, 1))
        self.lib.shim_hanging(self.p, _ip(cnt), _ip(mas), w.ctypes.data_as(C.POINTER(C.c_double)))
        return cnt, mas[:t], w[:t]


CONFIGS = [
    ("2d_q1", lambda: W.allen_cahn_amr_2d(refine=3, degree=1, min_level=1, max_level=6), 1),
    ("2d_q2", lambda: W.allen_cahn_amr_2d(refine=3, degree=2, min_level=1, max_level=5), 1),
    ("2d_q2_periodic", lambda: W.cahn_hilliard_amr(2, refine=3, degree=2, min_level=1, max_level=5), 1),
    ("3d_q1_periodic", lambda: W.cahn_hilliard_amr(3, refine=2, degree=1, min_level=1, max_level=4, size=16.0), 1),
    ("3d_q2_vector_dirichlet", lambda: W.eshelby_3d(refine=1, degree=2, size=8.0, n_incl=2), 0),
]


@pytest.mark.parametrize("name,make,field", CONFIGS, ids=[c[0] for c in CONFIGS])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_engine_mesh_matches_oracle_under_random_marks(shim, name, make, field, seed):
    wl = make()
    if wl.adaptivity is None:
        wl.adaptivity = dict(min_level=0, max_level=3, period=0, criteria=[])
    ad = wl.adaptivity
    m = wl.mesh
    o = po.Oracle(wl, adaptivity=ad)
    sub = (C.c_int * 3)(*[m.subdivisions[d] if d < m.dim else 1 for d in range(3)])
    per = (C.c_int * 3)(*[int(m.periodic[d]) if d < m.dim else 0 for d in range(3)])
    mesh = Mesh(shim, shim.shim_uniform(m.dim, m.degree, sub, per, m.global_refinement, ad["max_level"]))
    assert mesh.p
    nq = (m.degree + 1) ** m.dim
    rng = np.random.default_rng(seed)
    ncomp = 1 if wl.fields[field].field_type == 0 else m.dim
    levels_seen = set()
    for _ in range(5):
        cells = mesh.cells()
        assert np.array_equal(cells, o.cells())
        lev = cells[:, 0]
        marks = rng.choice([-1, 0, 1], size=len(cells), p=[0.45, 0.3, 0.25]).astype(np.int8)
        marks[(marks == 1) & (lev >= ad["max_level"])] = 0
        marks[(marks == -1) & (lev <= ad["min_level"])] = 0
        # a field to transfer (the oracle transfers it; the engine's plan must give the same)
        u = rng.uniform(-1.0, 1.0, ncomp * o.n_nodes())
        o.set_native(field, u)
        u = o.get_native(field)
        flags = marks.copy()
        new = Mesh(shim, shim.shim_refine(mesh.p, flags.ctypes.data_as(C.POINTER(C.c_byte)), ad["max_level"]))
        o.adapt_with_flags(marks.astype(np.int32))
        assert np.array_equal(new.cells(), o.cells())
        assert np.array_equal(new.cell_dofs(nq).astype(np.int64), o.cell_dofs(0))
        cnt, mas, w = new.hanging()
        ocnt, omas, ow = o.hanging()
        assert np.array_equal(cnt, ocnt) and np.array_equal(mas.astype(np.int64), omas) and np.array_equal(w, ow)
        # transfer plan, then the hanging lines, against the oracle's transferred field
        N, No = o.n_nodes(), len(u) // ncomp
        t = shim.shim_transfer(mesh.p, new.p, None, None, None)
        ptr, idx, tw = np.zeros(N + 1, np.int32), np.zeros(max(t, 1), np.int32), np.zeros(max(t, 1))
        shim.shim_transfer(mesh.p, new.p, _ip(ptr), _ip(idx), tw.ctypes.data_as(C.POINTER(C.c_double)))
        # then distribute as the engine does: Dirichlet rows take their values, hanging rows the
        # interpolant of their (free or Dirichlet) masters
        kind, _, inhom = o.constraints(field)
        got = np.zeros(ncomp * N)
        off = np.concatenate([[0], np.cumsum(cnt)])
        for c in range(ncomp):
            uc = u[c * No:(c + 1) * No]
            v = np.add.reduceat(tw[:t] * uc[idx[:t]], ptr[:-1]) if t else np.zeros(N)
            v[ptr[:-1] == ptr[1:]] = 0.0
            dir_rows = kind[c * N:(c + 1) * N].astype(bool) & (cnt == 0)
            v[dir_rows] = inhom[c * N:(c + 1) * N][dir_rows]
            for p in np.nonzero(cnt)[0]:
                v[p] = (w[off[p]:off[p + 1]] * v[mas[off[p]:off[p + 1]]]).sum()
            got[c * N:(c + 1) * N] = v
        ref = o.get_native(field)
        assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
        levels_seen.update(np.unique(new.cells()[:, 0]).tolist())
        shim.shim_free(mesh.p)
        mesh = new
    shim.shim_free(mesh.p)
    assert len(levels_seen) > 1
