// Allen-Cahn with a fixed grain table: n relaxes by dn/dt = -M (f'(n) - kappa lap n) with
// f'(n) = 4 n (n-1)(n-1/2), M = 1, kappa = 2. The initial n sums the tanh profiles (width
// GOLD_WIDTH) of the GOLD_N grains of "gold_ic.h" (centres and radii, written by the test from
// its fixture), capped at 1. Post-processing: |grad n| and n^4 - 2n^3 + n^2 + kappa/2 |grad n|^2.
#include <prismspf/core/pde_operator_base.h>

#include "gold_ic.h"

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim, unsigned int degree, typename number>
class CustomPDE : public PDEOperatorBase<dim, degree, number>
{
public:
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad  = dealii::Tensor<1, dim, ScalarValue>;

  CustomPDE(const UserInputParameters<dim> &_user_inputs, PhaseFieldTools<dim> &_pf_tools)
    : PDEOperatorBase<dim, degree, number>(_user_inputs, _pf_tools)
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
        variable_list.set_value_term(0, n - dt * mobility * fprime);
        variable_list.set_gradient_term(0, -dt * kappa * mobility * grad_n);
      }
    else if (solve_block_id == 2)
      {
        const ScalarValue n      = variable_list.template get_value<Scalar, Current>(0);
        const ScalarGrad  grad_n = variable_list.template get_gradient<Scalar, Current>(0);
        const ScalarValue f_chem = n * n * n * n - 2.0 * n * n * n + n * n;
        variable_list.set_value_term(1, grad_n.norm());
        variable_list.set_value_term(2, f_chem + 0.5 * kappa * grad_n.norm_square());
      }
  }

  number mobility = 1.0;
  number kappa    = 2.0;
};

PRISMS_PF_END_NAMESPACE
