// Elastic field of seeded misfitting inclusions: one vector field u solved by a Linear block
// (CG with the preconditioner from the parameter file) at increment 0.
#include "custom_pde.h"

#include <prismspf/core/parse_cmd_options.h>
#include <prismspf/core/problem.h>

using namespace prismspf;

int
main(int argc, char *argv[])
{
  prismspf::MPIInitFinalize mpi_init(argc, argv);
  ParseCMDOptions           cli_options(argc, argv);

  constexpr unsigned int dim    = 3;
  constexpr unsigned int degree = 2;

  std::vector<FieldAttributes> fields = {FieldAttributes("u", Vector)};

  SolveBlock elasticity;
  elasticity.id               = 1;
  elasticity.solve_type       = Linear;
  elasticity.solve_timing     = Uninitialized;
  elasticity.field_indices    = {0};
  elasticity.dependencies_rhs = make_dependency_set(fields, {});
  elasticity.dependencies_lhs = make_dependency_set(fields, {"grad(lhs(u))"});

  std::vector<SolveBlock> blocks({elasticity});

  UserInputParameters<dim>       user_inputs(cli_options.get_parameters_filename());
  PhaseFieldTools<dim>           pf_tools;
  CustomPDE<dim, degree, double> pde(user_inputs, pf_tools);
  Problem<dim, degree, double>   problem(fields, blocks, user_inputs, pf_tools, pde);
  problem.solve();
  return 0;
}
