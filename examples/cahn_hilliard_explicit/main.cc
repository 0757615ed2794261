// Cahn-Hilliard explicit application: c (Primary), mu (Secondary, solved after c every
// increment) and f_tot (post-processed on output increments).
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

  std::vector<FieldAttributes> fields = {FieldAttributes("c", Scalar),
                                         FieldAttributes("mu", Scalar),
                                         FieldAttributes("f_tot", Scalar)};

  SolveBlock concentration;
  concentration.id               = 0;
  concentration.solve_type       = Explicit;
  concentration.solve_timing     = Primary;
  concentration.field_indices    = {0};
  concentration.dependencies_rhs = make_dependency_set(fields, {"old_1(c)", "grad(old_1(mu))"});

  SolveBlock potential;
  potential.id               = 1;
  potential.solve_type       = Explicit;
  potential.solve_timing     = Secondary;
  potential.field_indices    = {1};
  potential.dependencies_rhs = make_dependency_set(fields, {"c", "grad(c)"});

  SolveBlock energy;
  energy.id               = 2;
  energy.solve_type       = Explicit;
  energy.solve_timing     = PostProcess;
  energy.field_indices    = {2};
  energy.dependencies_rhs = make_dependency_set(fields, {"c", "grad(c)"});

  std::vector<SolveBlock> blocks({concentration, potential, energy});

  UserInputParameters<dim>       user_inputs(cli_options.get_parameters_filename());
  PhaseFieldTools<dim>           pf_tools;
  CustomPDE<dim, degree, double> pde(user_inputs, pf_tools);
  Problem<dim, degree, double>   problem(fields, blocks, user_inputs, pf_tools, pde);
  problem.solve();
  return 0;
}
