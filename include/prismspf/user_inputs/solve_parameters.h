// Linear and nonlinear solver parameters of a solve block (reference:
// include/prismspf/user_inputs/solve_parameters.h, src/user_inputs/solve_parameters.cc:10-187).
#pragma once

#include <map>
#include <string>

#include <prismspf/config.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/core/types.h>

PRISMS_PF_BEGIN_NAMESPACE

// the members of PreconditionChebyshev::AdditionalData the solver reads
struct ChebyshevParameters {
  unsigned int degree = 5;
  double smoothing_range = 15.0;
  unsigned int eig_cg_n_iterations = 10;
};

struct LinearSolverParameters {
  std::string solver_type = "cg";
  double tolerance = 1.0e-10;
  SolverToleranceType tolerance_type = SolverToleranceType::RMSEPerField;
  unsigned int max_iterations = 100;
  unsigned int mg_depth = 1;
  PreconditionerType preconditioner = PreconditionerType::None;
  ChebyshevParameters chebyshev_parameters;
};

struct LinearSolveParameters {
  // solve-block id -> its parameters ("linear solver parameters: k" subsections)
  std::map<unsigned int, LinearSolverParameters> linear_solvers;
};

struct NonlinearSolverParameters {
  double step_length = 1.0;
  unsigned int max_iterations = 100;
  double tolerance_value = 1.0e-10;
};

struct NonlinearSolveParameters {
  std::map<Types::Index, NonlinearSolverParameters> nonlinear_solvers;
};

PRISMS_PF_END_NAMESPACE
