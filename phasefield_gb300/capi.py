"""ctypes bindings of the C ABI declared in ``include/ppf_gb300.h``.

The library is the in-tree ``phasefield_gb300/lib/libppf_gb300.so``. Loading fails loudly if it
is missing: there is no CPU fallback on the product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libppf_gb300.so"

PPF_MAX_FIELDS = 8
PPF_NAGE = 6

PPF_OK = 0
PPF_ERR_ARG = 1
PPF_ERR_NAN = 2
PPF_ERR_CUDA = 3
PPF_ERR_NOCONV = 4
PPF_ERR_DEPENDENCY = 5
PPF_ERR_UNSUPPORTED = 6
PPF_ERR_TIMEOUT = 7

ORDER_LATTICE = 0
ORDER_DEALII = 1
ORDER_NATIVE = 2

REFINE_VALUE = 1
REFINE_GRADIENT = 2

# exported symbols of include/ppf_gb300.h (checked by the CPU test suite)
EXPORTED = [
    "ppf_create", "ppf_destroy", "ppf_last_error", "ppf_n_nodes", "ppf_field_length", "ppf_n_cells",
    "ppf_dof_map", "ppf_constraint_map", "ppf_invm", "ppf_upload_state", "ppf_download_state",
    "ppf_apply_constraints", "ppf_run", "ppf_solve_block", "ppf_apply", "ppf_apply_device",
    "ppf_set_time", "ppf_get_time", "ppf_set_use_graph", "ppf_state_device_ptr", "ppf_synchronize",
    "ppf_set_stream", "ppf_kernel_timing", "ppf_kernel_stats", "ppf_kernel_stats_reset", "ppf_contraction_mode", "ppf_set_output_stream", "ppf_upload_state_async",
    "ppf_device_fp64_peak", "ppf_allen_cahn_step_noalloc", "ppf_allen_cahn_step_noalloc_status",
    "ppf_default_linear_params", "ppf_set_linear_params", "ppf_linear_solve", "ppf_lhs_diagonal",
    "ppf_set_newton_params", "ppf_newton_solve", "ppf_linear_stats", "ppf_increment_block", "ppf_end_increment",
    "ppf_set_nucleation_period", "ppf_upload_state_staged", "ppf_run_async", "ppf_wait",
    # ensembles (bound in phasefield_gb300/ensemble.py)
    "ppf_ensemble_create", "ppf_ensemble_destroy", "ppf_ensemble_last_error", "ppf_ensemble_instance_length",
    "ppf_ensemble_upload", "ppf_ensemble_download", "ppf_ensemble_run", "ppf_ensemble_autotune",
    "ppf_ensemble_synchronize", "ppf_ensemble_set_stream",
    "ppf_adjoint_forward", "ppf_adjoint_backward", "ppf_tangent_linear", "ppf_checkpoint_schedule_cost",
    # operators compiled by the caller (bound from C++ by prismspf/core/problem.h)
    "ppf_create_custom", "ppf_set_dirichlet_values", "ppf_dealii_cell_nodes", "ppf_download_solution",
    # adaptive meshes
    "ppf_set_adaptivity", "ppf_adapt", "ppf_remesh_if_due", "ppf_mesh_version", "ppf_cells", "ppf_cell_dofs",
    "ppf_node_points", "ppf_hanging", "ppf_set_dirichlet_function", "ppf_remesh_stats",
]


class MeshDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("degree", C.c_int), ("subdivisions", C.c_int * 3),
        ("lower", C.c_double * 3), ("size", C.c_double * 3), ("global_refinement", C.c_int),
        ("periodic", C.c_int * 3),
    ]


class FieldDesc(C.Structure):
    _fields_ = [
        ("rank", C.c_int), ("dirichlet", (C.c_int * 6) * 3), ("dirichlet_value", (C.c_double * 6) * 3),
    ]


class BlockDesc(C.Structure):
    _fields_ = [
        ("id", C.c_int), ("solve_type", C.c_int), ("solve_timing", C.c_int), ("n_fields", C.c_int),
        ("field_indices", C.c_int * PPF_MAX_FIELDS),
        ("dep_rhs", (C.c_ubyte * PPF_NAGE) * PPF_MAX_FIELDS),
        ("dep_lhs", (C.c_ubyte * PPF_NAGE) * PPF_MAX_FIELDS),
    ]


class LinearParams(C.Structure):
    _fields_ = [
        ("tolerance_type", C.c_int), ("tolerance", C.c_double), ("max_iterations", C.c_int),
        ("preconditioner", C.c_int), ("mg_depth", C.c_int), ("smoother_degree", C.c_int),
        ("smoothing_range", C.c_double), ("eig_cg_iterations", C.c_int), ("mixed_precision", C.c_int),
        ("solver_type", C.c_int),
    ]


class Adaptivity(C.Structure):
    _fields_ = [
        ("min_refinement", C.c_int),
        ("max_refinement", C.c_int),
        ("remeshing_period", C.c_int),
        ("n_criteria", C.c_int),
        ("criterion_field", C.c_int * PPF_MAX_FIELDS),
        ("criterion_flags", C.c_int * PPF_MAX_FIELDS),
        ("value_lower", C.c_double * PPF_MAX_FIELDS),
        ("value_upper", C.c_double * PPF_MAX_FIELDS),
        ("gradient_lower", C.c_double * PPF_MAX_FIELDS),
    ]


DIRICHLET_FN = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_double)


class PPFError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ppf error {code}: {msg}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    P = C.POINTER
    dp = P(C.c_double)
    H = C.c_void_p
    lib.ppf_create.argtypes = [P(MeshDesc), P(FieldDesc), C.c_int, P(BlockDesc), C.c_int, C.c_char_p, dp, C.c_int,
                               C.c_double, P(H)]
    lib.ppf_destroy.argtypes = [H]
    lib.ppf_destroy.restype = None
    lib.ppf_last_error.argtypes = [H]
    lib.ppf_last_error.restype = C.c_char_p
    for name in ("ppf_n_nodes", "ppf_n_cells"):
        getattr(lib, name).argtypes = [H]
        getattr(lib, name).restype = C.c_longlong
    lib.ppf_field_length.argtypes = [H, C.c_int]
    lib.ppf_field_length.restype = C.c_longlong
    lib.ppf_dof_map.argtypes = [H, C.c_int, P(C.c_longlong)]
    lib.ppf_constraint_map.argtypes = [H, C.c_int, P(C.c_int)]
    lib.ppf_invm.argtypes = [H, dp]
    lib.ppf_upload_state.argtypes = [H, C.c_int, C.c_int, dp, C.c_int]
    lib.ppf_download_state.argtypes = [H, C.c_int, C.c_int, dp, C.c_int]
    lib.ppf_apply_constraints.argtypes = [H, C.c_int]
    lib.ppf_run.argtypes = [H, C.c_uint, C.c_int]
    lib.ppf_solve_block.argtypes = [H, C.c_int]
    lib.ppf_apply.argtypes = [H, C.c_int, C.c_int, dp, dp, C.c_int]
    lib.ppf_apply_device.argtypes = [H, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    lib.ppf_set_time.argtypes = [H, C.c_uint, C.c_double]
    lib.ppf_get_time.argtypes = [H, P(C.c_uint), dp]
    lib.ppf_set_use_graph.argtypes = [H, C.c_int]
    lib.ppf_state_device_ptr.argtypes = [H, C.c_int, C.c_int, P(C.c_void_p)]
    lib.ppf_synchronize.argtypes = [H]
    lib.ppf_set_stream.argtypes = [H, C.c_void_p]
    lib.ppf_kernel_timing.argtypes = [H, C.c_int]
    lib.ppf_kernel_stats.argtypes = [H, dp, P(C.c_longlong), P(C.c_longlong)]
    lib.ppf_kernel_stats_reset.argtypes = [H]
    lib.ppf_contraction_mode.argtypes = [H, C.c_int, C.c_int, P(C.c_int)]
    lib.ppf_set_output_stream.argtypes = [H, C.c_int, dp, C.c_int]
    lib.ppf_upload_state_async.argtypes = [H, C.c_int, C.c_int, dp, C.c_int]
    lib.ppf_device_fp64_peak.argtypes = [dp]
    lib.ppf_allen_cahn_step_noalloc.argtypes = [P(MeshDesc), C.c_double, C.c_double, C.c_double, C.c_void_p,
                                                C.c_void_p, C.c_void_p]
    lib.ppf_allen_cahn_step_noalloc_status.argtypes = [C.c_void_p]
    lib.ppf_default_linear_params.argtypes = [P(LinearParams)]
    lib.ppf_set_linear_params.argtypes = [H, C.c_int, P(LinearParams)]
    lib.ppf_linear_solve.argtypes = [H, C.c_int, P(C.c_int), dp]
    lib.ppf_increment_block.argtypes = [H, C.c_int, C.c_int]
    lib.ppf_set_nucleation_period.argtypes = [H, C.c_uint]
    lib.ppf_upload_state_staged.argtypes = [H, C.c_int, C.c_int, dp]
    lib.ppf_run_async.argtypes = [H, C.c_uint, C.c_int]
    lib.ppf_wait.argtypes = [H]
    lib.ppf_end_increment.argtypes = [H]
    lib.ppf_linear_stats.argtypes = [H, C.c_int, dp, dp, dp, dp]
    lib.ppf_set_newton_params.argtypes = [H, C.c_int, C.c_int, C.c_double, C.c_double]
    lib.ppf_newton_solve.argtypes = [H, C.c_int, P(C.c_int), P(C.c_int), dp]
    lib.ppf_lhs_diagonal.argtypes = [H, C.c_int, dp]
    lib.ppf_adjoint_forward.argtypes = [H, C.c_int, C.c_int, C.c_int]
    lib.ppf_adjoint_backward.argtypes = [H, dp, dp, dp, P(C.c_longlong)]
    lib.ppf_tangent_linear.argtypes = [H, C.c_int, C.c_int, dp, dp, dp]
    lib.ppf_checkpoint_schedule_cost.argtypes = [C.c_int, C.c_int]
    lib.ppf_checkpoint_schedule_cost.restype = C.c_longlong
    lib.ppf_set_adaptivity.argtypes = [H, P(Adaptivity)]
    lib.ppf_adapt.argtypes = [H]
    lib.ppf_remesh_if_due.argtypes = [H]
    lib.ppf_mesh_version.argtypes = [H]
    lib.ppf_mesh_version.restype = C.c_longlong
    lib.ppf_cells.argtypes = [H, P(C.c_int)]
    lib.ppf_cell_dofs.argtypes = [H, P(C.c_int)]
    lib.ppf_node_points.argtypes = [H, dp]
    lib.ppf_hanging.argtypes = [H, P(C.c_int), P(C.c_int), dp]
    lib.ppf_hanging.restype = C.c_longlong
    lib.ppf_set_dirichlet_function.argtypes = [H, C.c_int, DIRICHLET_FN, C.c_void_p]
    lib.ppf_remesh_stats.argtypes = [H, dp]
    _lib = lib
    return lib


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))
