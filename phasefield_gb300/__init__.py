"""phasefield_gb300 — GB300-native matrix-free operator evaluation for PRISMS-PF problems.

The compute path is the CUDA library ``lib/libppf_gb300.so`` (C ABI in ``include/ppf_gb300.h``);
this package is its host-side mirror: problem description (fields, solve blocks, dependency
sets, mesh), seeded workloads, and the build step.
"""
from .capi import PPFError, load  # noqa: F401
from .problem import (Constant, Dependency, Explicit, FieldAttributes, Initialized, Linear, Newton,  # noqa: F401
                      NucleationRate, PostProcess, Primary, Problem, RectangularMesh, Scalar, Secondary,
                      SolveBlock, Uninitialized, Vector, make_dependency_set)

__all__ = ["Problem", "FieldAttributes", "SolveBlock", "RectangularMesh", "make_dependency_set", "PPFError", "load"]
