// Allen-Cahn grain coarsening, backward Euler through a Newton block: each increment solves
// R(n) = n_old - n - dt M f'(n) (value) - dt kappa M grad n (gradient) = 0 with the Jacobian
// (1 + dt M f''(n)) dn + dt kappa M grad dn, f(n) = n^2 (1-n)^2. The time step is not bound by
// the explicit stability limit. Initial condition: seeded circular grains (as the explicit
// example). Post-processing: |grad n| and the free-energy density.
#include <prismspf/core/pde_operator_base.h>

#include <random>
#include <vector>

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
  {
    const unsigned int n_grains = get_user_inputs().user_constants.get_int("n_grains");
    const auto        &size = get_user_inputs().spatial_discretization.rectangular_mesh.size;
    RNGEngine         &rng  = get_user_inputs().misc_parameters.rng;
    std::uniform_real_distribution<double> unit(0.0, 1.0);
    for (unsigned int g = 0; g < n_grains; ++g)
      {
        dealii::Point<dim> c;
        for (unsigned int d = 0; d < dim; ++d)
          c[d] = size[d] * unit(rng);
        centres.push_back(c);
        radii.push_back(5.0 + 10.0 * unit(rng));
      }
  }

private:
  void
  set_initial_condition(const unsigned int                  &index,
                        [[maybe_unused]] const unsigned int &component,
                        const dealii::Point<dim>            &point,
                        number                              &scalar_value,
                        [[maybe_unused]] number             &vector_component_value) const override
  {
    if (index != 0)
      return;
    double n = 0.0;
    for (size_t g = 0; g < centres.size(); ++g)
      n += 0.5 * (1.0 - std::tanh((point.distance(centres[g]) - radii[g]) / 2.0));
    scalar_value = std::min(n, 1.0);
  }

  void
  compute_rhs(FieldContainer<dim, degree, number> &variable_list,
              const SimulationTimer               &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    const double dt = sim_timer.get_timestep();
    if (solve_block_id == 1)
      {
        const ScalarValue n      = variable_list.template get_value<Scalar, Current>(0);
        const ScalarGrad  grad_n = variable_list.template get_gradient<Scalar, Current>(0);
        const ScalarValue n_old  = variable_list.template get_value<Scalar, OldOne>(0);
        const ScalarValue fprime = 4.0 * n * (n - 1.0) * (n - 0.5);
        variable_list.set_value_term(0, n_old - n - dt * mobility * fprime);
        variable_list.set_gradient_term(0, -dt * kappa * mobility * grad_n);
      }
    else if (solve_block_id == 2)
      {
        const ScalarValue n      = variable_list.template get_value<Scalar, Current>(0);
        const ScalarGrad  grad_n = variable_list.template get_gradient<Scalar, Current>(0);
        const ScalarValue f_bulk = n * n * n * n - 2.0 * n * n * n + n * n;
        variable_list.set_value_term(1, grad_n.norm());
        variable_list.set_value_term(2, f_bulk + 0.5 * kappa * grad_n.norm_square());
      }
  }

  void
  compute_lhs(FieldContainer<dim, degree, number> &variable_list,
              const SimulationTimer               &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    const double dt = sim_timer.get_timestep();
    if (solve_block_id == 1)
      {
        const ScalarValue n        = variable_list.template get_value<Scalar, Current>(0);
        const ScalarValue change   = variable_list.template get_value<Scalar, Change>(0);
        const ScalarGrad  change_x = variable_list.template get_gradient<Scalar, Change>(0);
        const ScalarValue fsecond  = 12.0 * n * (n - 1.0) + 2.0;
        variable_list.set_value_term(0, change * (1.0 + dt * mobility * fsecond));
        variable_list.set_gradient_term(0, dt * kappa * mobility * change_x);
      }
  }

  number mobility;
  number kappa;
  std::vector<dealii::Point<dim>> centres;
  std::vector<double>             radii;
};

PRISMS_PF_END_NAMESPACE
