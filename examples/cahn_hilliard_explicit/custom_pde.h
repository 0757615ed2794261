// Cahn-Hilliard spinodal decomposition, explicit Euler (the 3-D Cahn-Hilliard benchmark
// configuration): dc/dt = div(M grad mu), mu = f'(c) - kappa lap c with
// f(c) = W c^2 (1-c)^2 / 4, so f'(c) = W c (c-1)(c-1/2) (W = 4 gives f = c^2 (1-c)^2).
// Initial condition: c = c0 + amplitude * U(-1, 1) drawn per support point from the
// parameter file's random seed.
#include <prismspf/core/pde_operator_base.h>

#include <random>

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
    , mobility(get_user_inputs().user_constants.get_double("mobility"))
    , kappa(get_user_inputs().user_constants.get_double("kappa"))
    , well(get_user_inputs().user_constants.get_double("well_height"))
    , c0(get_user_inputs().user_constants.get_double("c0"))
    , amplitude(get_user_inputs().user_constants.get_double("amplitude"))
    , noise(-1.0, 1.0)
  {}

private:
  void
  set_initial_condition(const unsigned int                  &index,
                        [[maybe_unused]] const unsigned int &component,
                        [[maybe_unused]] const dealii::Point<dim> &point,
                        number                              &scalar_value,
                        [[maybe_unused]] number             &vector_component_value) const override
  {
    if (index == 0)
      scalar_value = c0 + amplitude * noise(get_user_inputs().misc_parameters.rng);
  }

  void
  compute_rhs(FieldContainer<dim, degree, number> &variable_list,
              const SimulationTimer               &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    if (solve_block_id == 0)
      {
        const ScalarValue c       = variable_list.template get_value<Scalar, OldOne>(0);
        const ScalarGrad  grad_mu = variable_list.template get_gradient<Scalar, OldOne>(1);
        variable_list.set_value_term(0, c);
        variable_list.set_gradient_term(0, -sim_timer.get_timestep() * mobility * grad_mu);
      }
    else if (solve_block_id == 1)
      {
        const ScalarValue c      = variable_list.template get_value<Scalar, Current>(0);
        const ScalarGrad  grad_c = variable_list.template get_gradient<Scalar, Current>(0);
        variable_list.set_value_term(1, well * c * (c - 1.0) * (c - 0.5));
        variable_list.set_gradient_term(1, kappa * grad_c);
      }
    else if (solve_block_id == 2)
      {
        const ScalarValue c      = variable_list.template get_value<Scalar, Current>(0);
        const ScalarGrad  grad_c = variable_list.template get_gradient<Scalar, Current>(0);
        const ScalarValue f_bulk = 0.25 * well * c * c * (1.0 - c) * (1.0 - c);
        variable_list.set_value_term(2, f_bulk + 0.5 * kappa * grad_c.norm_square());
      }
  }

  number mobility;
  number kappa;
  number well;
  number c0;
  number amplitude;
  mutable std::uniform_real_distribution<double> noise;
};

PRISMS_PF_END_NAMESPACE
