// Enumerations of the PRISMS-PF user API, same names and values as
// include/prismspf/core/type_enums.h and include/prismspf/core/solve_block.h:28-51
// of the reference, so application code that names them compiles unchanged.
#pragma once

#include <prismspf/config.h>

PRISMS_PF_BEGIN_NAMESPACE

enum SolveType { Constant, Explicit, Linear, Newton };

enum TensorRank { Undefined = -1, Scalar = 0, Vector = 1 };

enum ElasticityModel { Isotropic, Transverse, Orthotropic, Anisotropic };

enum DependencyType {
  DST = -2,
  SRC = -1,
  LHS = SRC,
  Solution = SRC,
  Trial = SRC,
  Change = SRC,
  Current = 0,
  OldOne,
  OldTwo,
  OldThree,
  OldFour
};

enum SolveTiming {
  Primary,
  Initialized = Primary,
  Secondary,
  Uninitialized = Secondary,
  PostProcess,
  NucleationRate
};

enum SolverToleranceType { AbsoluteResidual, RMSEPerField, IntegratedPerField, RMSETotal, IntegratedTotal };

enum PreconditionerType { None, Chebyshev, GMG };

PRISMS_PF_END_NAMESPACE
