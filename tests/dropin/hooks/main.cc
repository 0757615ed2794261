// Allen-Cahn with pre/post_solve_block hooks and a user stop: fields n, mg_n and f_tot, an
// explicit block for n and a post-processing block, on 2-D Q1 elements. The operator's hooks
// print every call and stop the run after the increment given by the model constant
// `stop_increment`.
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
  std::vector<SolveBlock> blocks;
  blocks.push_back(SolveBlock(1, Explicit, Primary, {0},
                              make_dependency_set(fields, {"old_1(n)", "grad(old_1(n))"})));
  blocks.push_back(SolveBlock(2, Explicit, PostProcess, {1, 2},
                              make_dependency_set(fields, {"n", "grad(n)"})));

  UserInputParameters<dim>       user_inputs(cli_options.get_parameters_filename());
  PhaseFieldTools<dim>           pf_tools;
  CustomPDE<dim, degree, double> pde(user_inputs, pf_tools);
  Problem<dim, degree, double>   problem(fields, blocks, user_inputs, pf_tools, pde);
  problem.solve();
  return 0;
}
