"""ORACLE — test infrastructure only. ctypes wrapper of the CPU restatement (oracle.cc).

Builds ``oracle/build/liboracle.so`` with g++ (OpenMP, -O3) on first use and mirrors a
phasefield_gb300 Workload in it so tests can compare GPU results with the restatement on
the same seeded inputs. Vectors cross this wrapper in lattice order; the oracle itself works
in deal.II DoF order and the wrapper permutes with the oracle's own lattice table.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.cc"
LIB = HERE / "build" / "liboracle.so"

MODEL_IDS = {"allen_cahn": 1, "cahn_hilliard": 2, "eshelby": 3, "coupled_acch": 4, "allen_cahn_implicit": 5,
             "cahn_hilliard_implicit": 6}


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                                 (HERE / "oracle.h").stat().st_mtime):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        P = C.POINTER
        dp = P(C.c_double)
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [C.c_int, C.c_int, P(C.c_int), dp, dp, C.c_int, P(C.c_int)]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        lib.orc_n_dofs.argtypes = [C.c_void_p, C.c_int]
        lib.orc_n_dofs.restype = C.c_long
        lib.orc_n_cells.argtypes = [C.c_void_p]
        lib.orc_n_cells.restype = C.c_long
        lib.orc_gl.argtypes = [C.c_int, dp, dp, dp]
        lib.orc_lattice.argtypes = [C.c_void_p, C.c_int, P(C.c_int)]
        lib.orc_cell_dofs.argtypes = [C.c_void_p, C.c_int, P(C.c_long)]
        lib.orc_cell_coords.argtypes = [C.c_void_p, P(C.c_int)]
        lib.orc_invm.argtypes = [C.c_void_p, C.c_int, dp]
        lib.orc_add_field.argtypes = [C.c_void_p, C.c_int]
        lib.orc_set_dirichlet.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double]
        lib.orc_add_block.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P(C.c_int), C.c_int, P(C.c_int),
                                      P(C.c_int)]
        lib.orc_finalize.argtypes = [C.c_void_p, C.c_int, dp, C.c_int, C.c_double]
        lib.orc_constraints.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_long), dp]
        lib.orc_set_vector.argtypes = [C.c_void_p, C.c_int, C.c_int, dp]
        lib.orc_get_vector.argtypes = [C.c_void_p, C.c_int, C.c_int, dp]
        lib.orc_set_time.argtypes = [C.c_void_p, C.c_uint, C.c_double]
        lib.orc_explicit_block.argtypes = [C.c_void_p, C.c_int]
        lib.orc_run.argtypes = [C.c_void_p, C.c_uint, C.c_int]
        lib.orc_apply.argtypes = [C.c_void_p, C.c_int, C.c_int, dp, dp, C.c_int]
        lib.orc_set_linear_params.argtypes = [C.c_void_p, C.c_int, dp]
        lib.orc_linear_solve.argtypes = [C.c_void_p, C.c_int, P(C.c_int), dp]
        lib.orc_diagonal.argtypes = [C.c_void_p, C.c_int, dp]
        lib.orc_increment_block.argtypes = [C.c_void_p, C.c_int, C.c_int]
        lib.orc_end_increment.argtypes = [C.c_void_p]
        lib.orc_set_nucleation_period.argtypes = [C.c_void_p, C.c_uint]
        lib.orc_set_solver_type.argtypes = [C.c_void_p, C.c_int, C.c_int]
        lib.orc_set_newton_params.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]
        lib.orc_newton_solve.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int), dp]
        lib.orc_set_adaptivity.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_int), P(C.c_int),
                                           dp, dp, dp]
        lib.orc_adapt.argtypes = [C.c_void_p]
        lib.orc_adapt_with_flags.argtypes = [C.c_void_p, P(C.c_int)]
        lib.orc_remesh_if_due.argtypes = [C.c_void_p]
        lib.orc_n_nodes.argtypes = [C.c_void_p]
        lib.orc_n_nodes.restype = C.c_long
        lib.orc_cells.argtypes = [C.c_void_p, P(C.c_int)]
        lib.orc_node_points.argtypes = [C.c_void_p, dp]
        lib.orc_hanging.argtypes = [C.c_void_p, P(C.c_int), P(C.c_long), dp]
        lib.orc_hanging.restype = C.c_long
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def gl_rule(n: int):
    lib = load()
    x, w, D = np.zeros(n), np.zeros(n), np.zeros(n * n)
    lib.orc_gl(n, _dp(x), _dp(w), _dp(D))
    return x, w, D.reshape(n, n)


class Oracle:
    """The workload's problem restated on the CPU."""

    def __init__(self, wl, threads: int = 0, adaptivity: dict | None = None):
        """adaptivity: {min_level, max_level, period, criteria: [(field, flags, vlo, vhi, glo)]}
        (flags 1 value, 2 gradient); the mesh starts uniform at the global refinement and the
        vectors of this wrapper are then in the adaptive DoF order (``*_native``)."""
        self.lib = load()
        self.wl = wl
        m = wl.mesh
        sub = (C.c_int * 3)(*[m.subdivisions[d] if d < m.dim else 1 for d in range(3)])
        lo = (C.c_double * 3)(*[m.lower[d] if d < m.dim else 0.0 for d in range(3)])
        sz = (C.c_double * 3)(*[m.size[d] if d < m.dim else 1.0 for d in range(3)])
        per = (C.c_int * 3)(*[int(m.periodic[d]) if d < m.dim else 0 for d in range(3)])
        self.h = self.lib.orc_create(m.dim, m.degree, sub, lo, sz, m.global_refinement, per)
        if not self.h:
            raise RuntimeError("oracle: bad mesh")
        if threads:
            self.lib.orc_set_threads(self.h, threads)
        from phasefield_gb300.problem import dep_table
        for fa in wl.fields:
            f = self.lib.orc_add_field(self.h, fa.field_type)
            for (comp, bid), val in fa.dirichlet.items():
                self.lib.orc_set_dirichlet(self.h, f, comp, bid, float(val))
        nf = len(wl.fields)
        for b in wl.blocks:
            fi = (C.c_int * len(b.field_indices))(*b.field_indices)
            tr = dep_table(b.dependencies_rhs)[:nf].astype(np.int32).ravel()
            tl = dep_table(b.dependencies_lhs)[:nf].astype(np.int32).ravel()
            self.lib.orc_add_block(self.h, b.id, b.solve_type, b.solve_timing, fi, len(b.field_indices),
                                   tr.ctypes.data_as(C.POINTER(C.c_int)), tl.ctypes.data_as(C.POINTER(C.c_int)))
        self.adaptive = adaptivity is not None
        if self.adaptive:
            # node positions are in units of the node spacing at max_level
            self._shift = int(adaptivity["max_level"]) - m.global_refinement
            crit = adaptivity.get("criteria", [])
            ci = lambda k: (C.c_int * max(1, len(crit)))(*[int(c[k]) for c in crit])
            cd = lambda k: (C.c_double * max(1, len(crit)))(*[float(c[k]) for c in crit])
            rc = self.lib.orc_set_adaptivity(self.h, int(adaptivity["min_level"]), int(adaptivity["max_level"]),
                                             int(adaptivity.get("period", 0)), len(crit), ci(0), ci(1), cd(2), cd(3),
                                             cd(4))
            if rc != 0:
                raise RuntimeError("oracle: adaptivity parameters rejected")
        consts = np.ascontiguousarray(np.asarray(wl.constants, dtype=np.float64))
        rc = self.lib.orc_finalize(self.h, MODEL_IDS[wl.model], _dp(consts), len(consts), float(wl.dt))
        if rc != 0:
            raise RuntimeError("oracle: finalize failed")
        self._perm = {}
        for f, v in wl.initial.items():
            if self.adaptive:
                self.set_native(f, self.lattice_to_native(f, v))
            else:
                self.set(f, v)

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- numbering ------------------------------------------------------------------------
    def n_dofs(self, rank: int) -> int:
        return int(self.lib.orc_n_dofs(self.h, rank))

    def lattice(self, rank: int) -> np.ndarray:
        n = self.n_dofs(rank)
        out = np.zeros((n, 4), dtype=np.int32)
        self.lib.orc_lattice(self.h, rank, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def dealii_to_lattice(self, rank: int) -> np.ndarray:
        """deal.II dof index -> lattice index (component-major)."""
        if rank not in self._perm:
            m = self.wl.mesh
            nn = m.nodes + [1] * (3 - m.dim)
            L = self.lattice(rank).astype(np.int64)
            N = int(np.prod(nn))
            self._perm[rank] = L[:, 3] * N + (L[:, 2] * nn[1] + L[:, 1]) * nn[0] + L[:, 0]
        return self._perm[rank]

    def cell_dofs(self, rank: int) -> np.ndarray:
        nloc = (self.wl.mesh.degree + 1) ** self.wl.mesh.dim * (1 if rank == 0 else self.wl.mesh.dim)
        out = np.zeros(int(self.lib.orc_n_cells(self.h)) * nloc, dtype=np.int64)
        self.lib.orc_cell_dofs(self.h, rank, out.ctypes.data_as(C.POINTER(C.c_long)))
        return out

    def constraints(self, f: int):
        n = self.n_dofs(self.wl.fields[f].field_type)
        kind = np.zeros(n, np.int32)
        master = np.zeros(n, np.int64)
        inhom = np.zeros(n)
        self.lib.orc_constraints(self.h, f, kind.ctypes.data_as(C.POINTER(C.c_int)),
                                 master.ctypes.data_as(C.POINTER(C.c_long)), _dp(inhom))
        return kind, master, inhom

    def invm(self, rank: int = 0) -> np.ndarray:
        """Inverse lumped mass in lattice order."""
        v = np.zeros(self.n_dofs(rank))
        self.lib.orc_invm(self.h, rank, _dp(v))
        out = np.zeros_like(v)
        out[self.dealii_to_lattice(rank)] = v
        return out

    # --- vectors (lattice order at this interface) ----------------------------------------
    def _rank(self, f: int) -> int:
        return self.wl.fields[f].field_type

    def set(self, f: int, lattice_values: np.ndarray, age: int = 0):
        p = self.dealii_to_lattice(self._rank(f))
        v = np.ascontiguousarray(np.asarray(lattice_values, dtype=np.float64)[p])
        if self.lib.orc_set_vector(self.h, f, age, _dp(v)) != 0:
            raise RuntimeError("oracle: age not stored")

    def get(self, f: int, age: int = 0) -> np.ndarray:
        p = self.dealii_to_lattice(self._rank(f))
        v = np.zeros(p.size)
        if self.lib.orc_get_vector(self.h, f, age, _dp(v)) != 0:
            raise RuntimeError("oracle: age not stored")
        out = np.zeros(p.size)
        out[p] = v
        return out

    # --- adaptive meshes (native = adaptive DoF order, vector fields component-major) -------
    def n_nodes(self) -> int:
        return int(self.lib.orc_n_nodes(self.h))

    def n_cells(self) -> int:
        return int(self.lib.orc_n_cells(self.h))

    def cells(self) -> np.ndarray:
        """Active cells in tree order: (level, i, j, k)."""
        out = np.zeros((self.n_cells(), 4), np.int32)
        self.lib.orc_cells(self.h, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def node_points(self) -> np.ndarray:
        out = np.zeros((self.n_nodes(), 3))
        self.lib.orc_node_points(self.h, _dp(out))
        return out

    def hanging(self):
        """Closed hanging-node lines of the scalar DoFs: (count per DoF, masters, weights)."""
        n = self.n_nodes()
        t = int(self.lib.orc_hanging(self.h, None, None, None))
        cnt = np.zeros(n, np.int32)
        mas = np.zeros(max(t, 1), np.int64)
        w = np.zeros(max(t, 1))
        self.lib.orc_hanging(self.h, cnt.ctypes.data_as(C.POINTER(C.c_int)), mas.ctypes.data_as(C.POINTER(C.c_long)),
                             _dp(w))
        return cnt, mas[:t], w[:t]

    def lattice_to_native(self, f: int, lattice_values: np.ndarray) -> np.ndarray:
        """A lattice-order vector of the initial uniform mesh in the adaptive DoF order."""
        m = self.wl.mesh
        nn = m.nodes + [1] * (3 - m.dim)
        L = self.lattice(self._rank(f)).astype(np.int64)
        I = L[:, :3] >> self._shift
        idx = L[:, 3] * int(np.prod(nn)) + (I[:, 2] * nn[1] + I[:, 1]) * nn[0] + I[:, 0]
        return np.asarray(lattice_values, dtype=np.float64)[idx]

    def set_native(self, f: int, values: np.ndarray, age: int = 0):
        v = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
        if self.lib.orc_set_vector(self.h, f, age, _dp(v)) != 0:
            raise RuntimeError("oracle: age not stored")

    def get_native(self, f: int, age: int = 0) -> np.ndarray:
        v = np.zeros(self.n_dofs(self._rank(f)))
        if self.lib.orc_get_vector(self.h, f, age, _dp(v)) != 0:
            raise RuntimeError("oracle: age not stored")
        return v

    def invm_native(self, rank: int = 0) -> np.ndarray:
        v = np.zeros(self.n_dofs(rank))
        self.lib.orc_invm(self.h, rank, _dp(v))
        return v

    def adapt(self):
        """One remesh pass (mark, smooth, refine/coarsen, transfer)."""
        if self.lib.orc_adapt(self.h) != 0:
            raise RuntimeError("oracle: mesh is not adaptive")

    def adapt_with_flags(self, flags):
        """One remesh pass from given marks per cell (1 refine, -1 coarsen, 0 keep)."""
        f = np.ascontiguousarray(np.asarray(flags, dtype=np.int32))
        if self.lib.orc_adapt_with_flags(self.h, f.ctypes.data_as(C.POINTER(C.c_int))) != 0:
            raise RuntimeError("oracle: mesh is not adaptive")

    def remesh_if_due(self):
        self.lib.orc_remesh_if_due(self.h)

    def set_time(self, increment: int, time: float):
        self.lib.orc_set_time(self.h, increment, time)

    def solve_block(self, b: int):
        self.lib.orc_explicit_block(self.h, b)

    def run(self, n_increments: int, output_every: int = 0) -> int:
        return int(self.lib.orc_run(self.h, n_increments, output_every))

    def increment_block(self, b: int, is_output: bool = False) -> int:
        return int(self.lib.orc_increment_block(self.h, b, int(is_output)))

    def end_increment(self) -> int:
        return int(self.lib.orc_end_increment(self.h))

    def set_nucleation_period(self, period: int):
        assert self.lib.orc_set_nucleation_period(self.h, period) == 0

    def set_linear_params(self, b: int, tolerance_type=0, tolerance=1e-10, max_iterations=100, preconditioner=0,
                          mg_depth=1, smoother_degree=5, smoothing_range=15.0, eig_cg_iterations=10, solver_type=0,
                          **_):
        p = np.array([tolerance_type, tolerance, max_iterations, preconditioner, mg_depth, smoother_degree,
                      smoothing_range, eig_cg_iterations], dtype=np.float64)
        self.lib.orc_set_linear_params(self.h, b, _dp(p))
        self.lib.orc_set_solver_type(self.h, b, int(solver_type))

    def set_newton_params(self, b: int, max_iterations=100, tolerance=1e-10, step_length=1.0):
        self.lib.orc_set_newton_params(self.h, b, int(max_iterations), float(tolerance), float(step_length))

    def newton_solve(self, b: int):
        """One Newton solve of block b: (rc, Newton iterations, Krylov iterations, residual)."""
        its, lin, res = C.c_int(), C.c_int(), C.c_double()
        rc = self.lib.orc_newton_solve(self.h, b, C.byref(its), C.byref(lin), C.byref(res))
        return rc, its.value, lin.value, res.value

    def linear_solve(self, b: int):
        its, res = C.c_int(), C.c_double()
        rc = self.lib.orc_linear_solve(self.h, b, C.byref(its), C.byref(res))
        return rc, its.value, res.value

    def diagonal(self, b: int) -> np.ndarray:
        f = self.wl.blocks[b].field_indices[0]
        p = self.dealii_to_lattice(self._rank(f))
        d = np.zeros(p.size)
        self.lib.orc_diagonal(self.h, b, _dp(d))
        out = np.zeros(p.size)
        out[p] = d
        return out

    def apply(self, b: int, which: int, src: np.ndarray | None, scale: int = 0) -> np.ndarray:
        blk = self.wl.blocks[b]
        perms = [self.dealii_to_lattice(self._rank(f)) for f in blk.field_indices]
        n = sum(p.size for p in perms)
        s = None
        if src is not None:
            parts, off = [], 0
            for p in perms:
                parts.append(np.asarray(src[off:off + p.size])[p])
                off += p.size
            s = np.ascontiguousarray(np.concatenate(parts))
        d = np.zeros(n)
        self.lib.orc_apply(self.h, b, which, _dp(s) if s is not None else None, _dp(d), scale)
        out, off = np.zeros(n), 0
        for p in perms:
            seg = np.zeros(p.size)
            seg[p] = d[off:off + p.size]
            out[off:off + p.size] = seg
            off += p.size
        return out
