"""Host-side mirror of the PRISMS-PF problem-description API over the C ABI.

Names and meaning follow the reference: ``FieldAttributes`` (include/prismspf/core/field_attributes.h),
``SolveBlock`` (include/prismspf/core/solve_block.h:56-127), ``make_dependency_set``
(include/prismspf/core/dependencies.h:134-213, same dependency-string grammar: ``n``,
``grad(n)``, ``hess(n)``, ``lap(n)``, ``hessdiag(n)``, ``div(u)``, ``symgrad(u)``, ``curl(u)``,
``old_k(...)`` and ``src(...)/change(...)/trial(...)/lhs(...)``), and ``Problem``
(include/prismspf/core/problem.h) whose ``solve`` runs the increment loop of
src/core/problem.cc:341-557 on the GPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field as dfield

import numpy as np

from . import capi

# enums (include/prismspf/core/type_enums.h, solve_block.h)
Scalar, Vector = 0, 1
Constant, Explicit, Linear, Newton = 0, 1, 2, 3
Primary = Initialized = 0
Secondary = Uninitialized = 1
PostProcess = 2
NucleationRate = 3

VALUES, GRADIENTS, HESSIANS = 1, 2, 4
AGE_CURRENT, AGE_SRC = 0, 5


@dataclass
class FieldAttributes:
    name: str
    field_type: int = Scalar
    # {(component, boundary_id): value} Dirichlet conditions (constraint_parameters.cc:41-107)
    dirichlet: dict = dfield(default_factory=dict)


@dataclass
class Dependency:
    flag: int = 0
    src_flag: int = 0
    old_flags: list = dfield(default_factory=list)


def make_dependency_set(fields: list[FieldAttributes], dependency_strings, max_checked_age: int = 6) -> dict:
    """Parses dependency strings into {field_index: Dependency}; unknown strings raise."""
    reg = [("", "", VALUES), ("grad(", ")", GRADIENTS), ("hess(", ")", HESSIANS), ("hessdiag(", ")", HESSIANS),
           ("lap(", ")", HESSIANS), ("div(", ")", GRADIENTS), ("symgrad(", ")", GRADIENTS), ("curl(", ")", GRADIENTS)]
    srcs = [("src(", ")"), ("change(", ")"), ("trial(", ")"), ("lhs(", ")")]
    remaining = set(dependency_strings)
    result: dict[int, Dependency] = {}
    for i, attr in enumerate(fields):
        for pre, post, flag in reg:
            s = pre + attr.name + post
            if s in remaining:
                result.setdefault(i, Dependency()).flag |= flag
                remaining.discard(s)
            for s1, s2 in srcs:
                s = pre + s1 + attr.name + s2 + post
                if s in remaining:
                    result.setdefault(i, Dependency()).src_flag |= flag
                    remaining.discard(s)
            for age in range(max_checked_age):
                s = f"{pre}old_{age + 1}({attr.name}){post}"
                if s in remaining:
                    d = result.setdefault(i, Dependency())
                    while len(d.old_flags) < age + 1:
                        d.old_flags.append(0)
                    d.old_flags[age] |= flag
                    remaining.discard(s)
    if remaining:
        raise ValueError("The following dependencies were not recognized: " + ", ".join(sorted(remaining)))
    return result


@dataclass
class SolveBlock:
    id: int = 0
    solve_type: int = Explicit
    solve_timing: int = Primary
    field_indices: list = dfield(default_factory=list)
    dependencies_rhs: dict = dfield(default_factory=dict)
    dependencies_lhs: dict = dfield(default_factory=dict)


@dataclass
class RectangularMesh:
    dim: int
    degree: int
    size: tuple
    subdivisions: tuple = (1, 1, 1)
    lower: tuple = (0.0, 0.0, 0.0)
    global_refinement: int = 0
    periodic: tuple = (0, 0, 0)

    @property
    def cells(self) -> list[int]:
        return [self.subdivisions[d] << self.global_refinement for d in range(self.dim)]

    @property
    def nodes(self) -> list[int]:
        return [self.degree * c + 1 for c in self.cells]


def dep_table(deps: dict) -> np.ndarray:
    """{field: Dependency} -> [field][age] flag table (ages current, old_1..old_4, src)."""
    t = np.zeros((capi.PPF_MAX_FIELDS, capi.PPF_NAGE), dtype=np.uint8)
    for f, d in deps.items():
        t[f, AGE_CURRENT] |= d.flag
        t[f, AGE_SRC] |= d.src_flag
        for a, fl in enumerate(d.old_flags[:4]):
            t[f, 1 + a] |= fl
    return t


class Problem:
    """GPU problem handle: fields, solve blocks, mesh and a compiled operator set."""

    def __init__(self, fields: list[FieldAttributes], blocks: list[SolveBlock], mesh: RectangularMesh,
                 model: str, constants, dt: float):
        self.lib = capi.load()
        self.fields, self.blocks, self.mesh = fields, blocks, mesh
        m = capi.MeshDesc()
        m.dim, m.degree, m.global_refinement = mesh.dim, mesh.degree, mesh.global_refinement
        for d in range(3):
            m.subdivisions[d] = mesh.subdivisions[d] if d < mesh.dim else 1
            m.lower[d] = mesh.lower[d] if d < mesh.dim else 0.0
            m.size[d] = mesh.size[d] if d < mesh.dim else 1.0
            m.periodic[d] = int(mesh.periodic[d]) if d < mesh.dim else 0
        fds = (capi.FieldDesc * len(fields))()
        for i, fa in enumerate(fields):
            fds[i].rank = fa.field_type
            for (comp, bid), val in fa.dirichlet.items():
                fds[i].dirichlet[comp][bid] = 1
                fds[i].dirichlet_value[comp][bid] = float(val)
        bds = (capi.BlockDesc * max(1, len(blocks)))()
        for i, b in enumerate(blocks):
            bd = bds[i]
            bd.id, bd.solve_type, bd.solve_timing = b.id, b.solve_type, b.solve_timing
            bd.n_fields = len(b.field_indices)
            for j, f in enumerate(b.field_indices):
                bd.field_indices[j] = f
            tr, tl = dep_table(b.dependencies_rhs), dep_table(b.dependencies_lhs)
            for f in range(capi.PPF_MAX_FIELDS):
                for a in range(capi.PPF_NAGE):
                    bd.dep_rhs[f][a] = int(tr[f, a])
                    bd.dep_lhs[f][a] = int(tl[f, a])
        consts = np.ascontiguousarray(np.asarray(constants, dtype=np.float64))
        h = C.c_void_p()
        rc = self.lib.ppf_create(C.byref(m), fds, len(fields), bds, len(blocks), model.encode(), capi.dptr(consts),
                                 len(consts), float(dt), C.byref(h))
        if rc != capi.PPF_OK:
            raise capi.PPFError(rc, self.lib.ppf_last_error(None).decode())
        self.h = h

    # --- lifetime -------------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.ppf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != capi.PPF_OK:
            raise capi.PPFError(rc, self.lib.ppf_last_error(self.h).decode())

    def set_output_stream(self, f: int, host=None):
        """Stream field f into `host` (a float64 array of field_length(f), lattice order; pinned
        memory makes the copy asynchronous) after every increment, overlapping the copy with the
        blocks solved after f's (ppf_set_output_stream); None stops it."""
        streams = getattr(self, "_streams", {})
        if host is None:
            self._check(self.lib.ppf_set_output_stream(self.h, f, None, capi.ORDER_LATTICE))
            streams.pop(f, None)
            self._streams = streams
            return
        ptr = host.data_ptr() if hasattr(host, "data_ptr") else host.ctypes.data
        n = host.numel() if hasattr(host, "numel") else host.size
        if n != self.field_length(f):
            raise ValueError("host buffer length differs from the field length")
        self._check(self.lib.ppf_set_output_stream(self.h, f, C.cast(ptr, C.POINTER(C.c_double)), capi.ORDER_LATTICE))
        streams[f] = host  # the engine writes into it until streaming stops
        self._streams = streams

    def contraction_mode(self, block: int, which: int = 0) -> int:
        """0 FP64 contractions, 1 fixed-point derivatives with FP64 integration, 2 both in fixed
        point, 3 FP64 derivatives with fixed-point integration, 4 the lane kernel (every
        contraction and the value terms in fixed point, cubic cells), -1 not chosen yet
        (ppf_contraction_mode)."""
        m = C.c_int()
        self._check(self.lib.ppf_contraction_mode(self.h, block, which, C.byref(m)))
        return m.value

    # --- sizes ----------------------------------------------------------------------------
    @property
    def n_nodes(self) -> int:
        return int(self.lib.ppf_n_nodes(self.h))

    def field_length(self, f: int) -> int:
        return int(self.lib.ppf_field_length(self.h, f))

    # --- maps -----------------------------------------------------------------------------
    def dof_map(self, rank: int) -> np.ndarray:
        n = self.n_nodes * (1 if rank == 0 else self.mesh.dim)
        out = np.empty(n, dtype=np.int64)
        self._check(self.lib.ppf_dof_map(self.h, rank, out.ctypes.data_as(C.POINTER(C.c_longlong))))
        return out

    def constraint_map(self, f: int) -> np.ndarray:
        out = np.empty(self.field_length(f), dtype=np.int32)
        self._check(self.lib.ppf_constraint_map(self.h, f, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def invm(self) -> np.ndarray:
        out = np.empty(self.n_nodes, dtype=np.float64)
        self._check(self.lib.ppf_invm(self.h, capi.dptr(out)))
        return out

    # --- state ----------------------------------------------------------------------------
    def _io_length(self, f: int, ordering: int) -> int:
        # lattice-order vectors keep the initial lattice's length on adaptive meshes too
        if ordering == capi.ORDER_NATIVE or not getattr(self, "adaptive", False):
            return self.field_length(f)
        ncomp = 1 if self.fields[f].field_type == 0 else self.mesh.dim
        return ncomp * int(np.prod(self.mesh.nodes))

    def upload(self, f: int, values: np.ndarray, age: int = 0, ordering: int = capi.ORDER_LATTICE):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        if v.size != self._io_length(f, ordering):
            raise ValueError("wrong vector length")
        self._check(self.lib.ppf_upload_state(self.h, f, age, capi.dptr(v), ordering))

    def download(self, f: int, age: int = 0, ordering: int = capi.ORDER_LATTICE) -> np.ndarray:
        out = np.empty(self._io_length(f, ordering), dtype=np.float64)
        self._check(self.lib.ppf_download_state(self.h, f, age, capi.dptr(out), ordering))
        return out

    def download_solution(self, f: int, ordering: int = capi.ORDER_LATTICE) -> np.ndarray:
        """The field's solution after the last increment (ppf_download_solution)."""
        out = np.empty(self._io_length(f, ordering), dtype=np.float64)
        self._check(self.lib.ppf_download_solution(self.h, f, capi.dptr(out), ordering))
        return out

    # --- adaptive meshes --------------------------------------------------------------------
    def set_adaptivity(self, adaptivity: dict):
        """{min_level, max_level, period, criteria: [(field, flags, vlo, vhi, glo)]} (flags 1 value,
        2 gradient); the mesh starts uniform at the global refinement (ppf_set_adaptivity)."""
        a = capi.Adaptivity()
        a.min_refinement = int(adaptivity["min_level"])
        a.max_refinement = int(adaptivity["max_level"])
        a.remeshing_period = int(adaptivity.get("period", 0))
        crit = adaptivity.get("criteria", [])
        a.n_criteria = len(crit)
        for i, (f, fl, vlo, vhi, glo) in enumerate(crit):
            a.criterion_field[i], a.criterion_flags[i] = int(f), int(fl)
            a.value_lower[i], a.value_upper[i], a.gradient_lower[i] = float(vlo), float(vhi), float(glo)
        self._check(self.lib.ppf_set_adaptivity(self.h, C.byref(a)))
        self.adaptive = True

    def adapt(self):
        self._check(self.lib.ppf_adapt(self.h))

    def remesh_if_due(self):
        self._check(self.lib.ppf_remesh_if_due(self.h))

    def remesh_stats(self) -> dict:
        """Phases of the last remeshing pass in ms (ppf_remesh_stats)."""
        v = np.zeros(5)
        self._check(self.lib.ppf_remesh_stats(self.h, capi.dptr(v)))
        return dict(zip(("criteria_ms", "smoothing_ms", "new_mesh_ms", "transfer_ms", "setup_ms"), v.tolist()))

    @property
    def mesh_version(self) -> int:
        return int(self.lib.ppf_mesh_version(self.h))

    @property
    def n_cells(self) -> int:
        return int(self.lib.ppf_n_cells(self.h))

    def cells(self) -> np.ndarray:
        """Active cells: (level, x, y, z) each, tree order on adaptive meshes."""
        out = np.empty((self.n_cells, 4), dtype=np.int32)
        self._check(self.lib.ppf_cells(self.h, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def cell_dofs(self) -> np.ndarray:
        out = np.empty(self.n_cells * (self.mesh.degree + 1) ** self.mesh.dim, dtype=np.int32)
        self._check(self.lib.ppf_cell_dofs(self.h, out.ctypes.data_as(C.POINTER(C.c_int))))
        return out

    def node_points(self) -> np.ndarray:
        out = np.empty((self.n_nodes, 3), dtype=np.float64)
        self._check(self.lib.ppf_node_points(self.h, capi.dptr(out)))
        return out

    def hanging(self):
        """Closed hanging-node lines: (count per DoF, masters, weights)."""
        t = int(self.lib.ppf_hanging(self.h, None, None, None))
        cnt = np.empty(self.n_nodes, dtype=np.int32)
        mas = np.empty(max(t, 1), dtype=np.int32)
        w = np.empty(max(t, 1), dtype=np.float64)
        self.lib.ppf_hanging(self.h, cnt.ctypes.data_as(C.POINTER(C.c_int)), mas.ctypes.data_as(C.POINTER(C.c_int)),
                             capi.dptr(w))
        return cnt, mas[:t], w[:t]

    def apply_constraints(self, f: int):
        self._check(self.lib.ppf_apply_constraints(self.h, f))

    # --- solves ---------------------------------------------------------------------------
    def solve(self, n_increments: int, output_every: int = 0):
        """Problem::solve: increments from the current one through n_increments."""
        self._check(self.lib.ppf_run(self.h, n_increments, output_every))

    def set_nucleation_period(self, period: int):
        """NucleationRate blocks also run on increments divisible by `period`."""
        self._check(self.lib.ppf_set_nucleation_period(self.h, period))

    def increment_block(self, b: int, is_output: bool = False):
        """Block b's part of the current increment (ppf_increment_block)."""
        self._check(self.lib.ppf_increment_block(self.h, b, int(is_output)))

    def end_increment(self):
        """Age rotation and timer advance at the end of an increment (ppf_end_increment)."""
        self._check(self.lib.ppf_end_increment(self.h))

    def device_view(self, f: int, age: int = 0):
        """The device vector of field f at `age` as a torch CUDA tensor (no copy). Valid until
        the next age rotation or the next run that consumes a staged upload of the field; the
        caller orders its work with the handle's stream."""
        import torch
        ptr = C.c_void_p()
        self._check(self.lib.ppf_state_device_ptr(self.h, f, age, C.byref(ptr)))
        n = self.field_length(f)

        class _View:
            __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr.value, False), "version": 3}
        return torch.as_tensor(_View(), device="cuda")

    def solve_block(self, b: int):
        self._check(self.lib.ppf_solve_block(self.h, b))

    def apply(self, b: int, which: int, src: np.ndarray | None, scale: int = 0) -> np.ndarray:
        n = sum(self.field_length(f) for f in self.blocks[b].field_indices)
        dst = np.empty(n, dtype=np.float64)
        sp = None
        if src is not None:
            src = np.ascontiguousarray(src, dtype=np.float64)
            sp = capi.dptr(src)
        self._check(self.lib.ppf_apply(self.h, b, which, sp, capi.dptr(dst), scale))
        return dst

    # --- linear solves --------------------------------------------------------------------
    def set_linear_params(self, b: int, **kw):
        """LinearSolverParameters of Linear block b (keys of ppf_linear_params)."""
        p = capi.LinearParams()
        self.lib.ppf_default_linear_params(C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        self._check(self.lib.ppf_set_linear_params(self.h, b, C.byref(p)))

    def linear_solve(self, b: int, allow_noconv: bool = False) -> tuple[int, float]:
        its, res = C.c_int(), C.c_double()
        rc = self.lib.ppf_linear_solve(self.h, b, C.byref(its), C.byref(res))
        if rc == capi.PPF_ERR_NOCONV and allow_noconv:
            return its.value, res.value
        self._check(rc)
        return its.value, res.value

    def linear_stats(self, b: int) -> dict:
        """Wall-clock phases (ms) of the last linear solve of block b."""
        z, a, r, i = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.ppf_linear_stats(self.h, b, C.byref(z), C.byref(a), C.byref(r), C.byref(i)))
        return {"init_ms": z.value, "setup_ms": a.value, "rhs_ms": r.value, "iterate_ms": i.value}

    def set_newton_params(self, b: int, max_iterations: int = 100, tolerance: float = 1e-10,
                          step_length: float = 1.0):
        """NonlinearSolverParameters of Newton block b."""
        self._check(self.lib.ppf_set_newton_params(self.h, b, int(max_iterations), float(tolerance),
                                                   float(step_length)))

    def newton_solve(self, b: int, allow_noconv: bool = False) -> tuple[int, int, float]:
        """One Newton solve of block b: (Newton iterations, Krylov iterations, residual)."""
        its, lin, res = C.c_int(), C.c_int(), C.c_double()
        rc = self.lib.ppf_newton_solve(self.h, b, C.byref(its), C.byref(lin), C.byref(res))
        if not (rc == capi.PPF_ERR_NOCONV and allow_noconv):
            self._check(rc)
        return its.value, lin.value, res.value

    def lhs_diagonal(self, b: int) -> np.ndarray:
        f = self.blocks[b].field_indices[0]
        out = np.empty(self.field_length(f), dtype=np.float64)
        self._check(self.lib.ppf_lhs_diagonal(self.h, b, capi.dptr(out)))
        return out

    # --- adjoint (coupled_acch explicit block) --------------------------------------------
    def adjoint_forward(self, b: int, n_steps: int, n_snapshots: int):
        self._check(self.lib.ppf_adjoint_forward(self.h, b, n_steps, n_snapshots))

    def adjoint_backward(self, dJ_duK: np.ndarray):
        """Returns (dJ/d(Mc, Kn), dJ/du_0, forward steps taken)."""
        g = np.ascontiguousarray(dJ_duK, dtype=np.float64)
        dp = np.zeros(2)
        du0 = np.zeros_like(g)
        steps = C.c_longlong()
        self._check(self.lib.ppf_adjoint_backward(self.h, capi.dptr(g), capi.dptr(dp), capi.dptr(du0),
                                                  C.byref(steps)))
        return dp, du0, steps.value

    def tangent_linear(self, b: int, n_steps: int, du0: np.ndarray, dparams) -> np.ndarray:
        d0 = np.ascontiguousarray(du0, dtype=np.float64)
        dp = np.ascontiguousarray(dparams, dtype=np.float64)
        out = np.zeros_like(d0)
        self._check(self.lib.ppf_tangent_linear(self.h, b, n_steps, capi.dptr(d0), capi.dptr(dp), capi.dptr(out)))
        return out

    def set_time(self, increment: int, time: float):
        self._check(self.lib.ppf_set_time(self.h, increment, time))

    def get_time(self) -> tuple[int, float]:
        inc, t = C.c_uint(), C.c_double()
        self._check(self.lib.ppf_get_time(self.h, C.byref(inc), C.byref(t)))
        return inc.value, t.value

    def synchronize(self):
        self._check(self.lib.ppf_synchronize(self.h))
