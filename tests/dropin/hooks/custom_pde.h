// Allen-Cahn (as tests/dropin/gold_3_6, initial grains from "gold_ic.h") with the solve-block
// hooks of PDEOperatorBase overridden: each call prints "hook <pre|post> <block id> <increment>
// <time>", the post hook of block 1 also prints the sum of n read through the SolveContext, and
// at increment `stop_increment` it calls set_user_stop(true).
#include <prismspf/core/pde_operator_base.h>

#include <cstdio>

#include "gold_ic.h"

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim, unsigned int degree, typename number>
class CustomPDE : public PDEOperatorBase<dim, degree, number>
{
public:
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad  = dealii::Tensor<1, dim, ScalarValue>;
  using PDEOperatorBase<dim, degree, number>::get_user_inputs;

  CustomPDE(const UserInputParameters<dim> &_user_inputs, PhaseFieldTools<dim> &_pf_tools)
    : PDEOperatorBase<dim, degree, number>(_user_inputs, _pf_tools)
    , stop_increment(get_user_inputs().user_constants.get_int("stop_increment"))
  {}

private:
  void
  set_initial_condition(const unsigned int       &index,
                        [[maybe_unused]] const unsigned int &component,
                        const dealii::Point<dim> &point,
                        number                   &scalar_value,
                        [[maybe_unused]] number  &vector_component_value) const override
  {
    if (index != 0)
      return;
    for (int g = 0; g < GOLD_N; ++g)
      {
        double r2 = 0.0;
        for (unsigned int d = 0; d < dim; ++d)
          r2 += (point[d] - gold_centres[g][d]) * (point[d] - gold_centres[g][d]);
        scalar_value += 0.5 * (1.0 - std::tanh((std::sqrt(r2) - gold_radii[g]) / GOLD_WIDTH));
      }
    scalar_value = std::min(scalar_value, static_cast<number>(1.0));
  }

  void
  compute_rhs(FieldContainer<dim, degree, number> &variable_list,
              const SimulationTimer               &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    if (solve_block_id == 1)
      {
        const ScalarValue n      = variable_list.template get_value<Scalar, OldOne>(0);
        const ScalarGrad  grad_n = variable_list.template get_gradient<Scalar, OldOne>(0);
        const ScalarValue fprime = 4.0 * n * (n - 1.0) * (n - 0.5);
        const double      dt     = sim_timer.get_timestep();
        variable_list.set_value_term(0, n - dt * fprime);
        variable_list.set_gradient_term(0, -dt * 2.0 * grad_n);
      }
    else if (solve_block_id == 2)
      {
        const ScalarValue n      = variable_list.template get_value<Scalar, Current>(0);
        const ScalarGrad  grad_n = variable_list.template get_gradient<Scalar, Current>(0);
        const ScalarValue f_chem = n * n * n * n - 2.0 * n * n * n + n * n;
        variable_list.set_value_term(1, grad_n.norm());
        variable_list.set_value_term(2, f_chem + grad_n.norm_square());
      }
  }

  void
  pre_solve_block(SolveContext<dim, degree, number> &solve_context, unsigned int solver_id) override
  {
    const SimulationTimer &t = solve_context.get_simulation_timer();
    std::printf("hook pre %u %u %.4f\n", solver_id, t.get_increment(), t.get_time());
  }

  void
  post_solve_block(SolveContext<dim, degree, number> &solve_context, unsigned int solver_id) override
  {
    const SimulationTimer &t = solve_context.get_simulation_timer();
    std::printf("hook post %u %u %.4f\n", solver_id, t.get_increment(), t.get_time());
    if (solver_id == 1)
      {
        double sum = 0.0;
        for (double v : solve_context.get_solution(0))
          sum += v;
        std::printf("hook sum %u %.17g\n", t.get_increment(), sum);
        if ((int)t.get_increment() == stop_increment)
          this->set_user_stop(true);
      }
    std::fflush(stdout);
  }

  int stop_increment;
};

PRISMS_PF_END_NAMESPACE
