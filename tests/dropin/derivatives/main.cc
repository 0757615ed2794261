// Test application for the derivative getters (see custom_pde.h).
#include "custom_pde.h"

#include <prismspf/core/parse_cmd_options.h>
#include <prismspf/core/problem.h>

using namespace prismspf;

int
main(int argc, char *argv[])
{
  prismspf::MPIInitFinalize mpi_init(argc, argv);
  ParseCMDOptions           cli_options(argc, argv);

  constexpr unsigned int dim    = 2;
  constexpr unsigned int degree = 2;

  std::vector<FieldAttributes> fields = {
    FieldAttributes("u", Scalar),      FieldAttributes("w", Vector),        FieldAttributes("lap_u", Scalar),
    FieldAttributes("hess_u", Scalar), FieldAttributes("div_w", Scalar),    FieldAttributes("curl_w", Scalar),
    FieldAttributes("sym_w_xy", Scalar), FieldAttributes("x_plus_vol", Scalar)};

  SolveBlock inputs;
  inputs.id            = 1;
  inputs.solve_type    = Constant;
  inputs.solve_timing  = Primary;
  inputs.field_indices = {0, 1};

  SolveBlock scalar_derivatives;
  scalar_derivatives.id               = 2;
  scalar_derivatives.solve_type       = Explicit;
  scalar_derivatives.solve_timing     = PostProcess;
  scalar_derivatives.field_indices    = {2, 3, 4};
  scalar_derivatives.dependencies_rhs = make_dependency_set(fields, {"hess(u)", "hessdiag(u)", "lap(u)", "div(w)"});

  SolveBlock vector_derivatives;
  vector_derivatives.id               = 3;
  vector_derivatives.solve_type       = Explicit;
  vector_derivatives.solve_timing     = PostProcess;
  vector_derivatives.field_indices    = {5, 6, 7};
  vector_derivatives.dependencies_rhs = make_dependency_set(fields, {"curl(w)", "symgrad(w)"});

  std::vector<SolveBlock> blocks({inputs, scalar_derivatives, vector_derivatives});

  UserInputParameters<dim>       user_inputs(cli_options.get_parameters_filename());
  PhaseFieldTools<dim>           pf_tools;
  CustomPDE<dim, degree, double> pde(user_inputs, pf_tools);
  Problem<dim, degree, double>   problem(fields, blocks, user_inputs, pf_tools, pde);
  problem.solve();
  return 0;
}
