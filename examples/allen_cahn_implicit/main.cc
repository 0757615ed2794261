// Implicit Allen-Cahn application: n solved by a Newton block every increment, mg_n and
// f_tot post-processed on output increments.
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
  constexpr unsigned int degree = 1;

  std::vector<FieldAttributes> fields = {FieldAttributes("n", Scalar),
                                         FieldAttributes("mg_n", Scalar),
                                         FieldAttributes("f_tot", Scalar)};

  SolveBlock evolve;
  evolve.id               = 1;
  evolve.solve_type       = Newton;
  evolve.solve_timing     = Primary;
  evolve.field_indices    = {0};
  evolve.dependencies_rhs = make_dependency_set(fields, {"n", "grad(n)", "old_1(n)"});
  evolve.dependencies_lhs = make_dependency_set(fields, {"n", "change(n)", "grad(change(n))"});

  SolveBlock post;
  post.id               = 2;
  post.solve_type       = Explicit;
  post.solve_timing     = PostProcess;
  post.field_indices    = {1, 2};
  post.dependencies_rhs = make_dependency_set(fields, {"n", "grad(n)"});

  std::vector<SolveBlock> blocks({evolve, post});

  UserInputParameters<dim>       user_inputs(cli_options.get_parameters_filename());
  PhaseFieldTools<dim>           pf_tools;
  CustomPDE<dim, degree, double> pde(user_inputs, pf_tools);
  Problem<dim, degree, double>   problem(fields, blocks, user_inputs, pf_tools, pde);
  problem.solve();
  return 0;
}
