// Allen-Cahn grain coarsening, explicit Euler (the 2-D Allen-Cahn benchmark configuration):
// n relaxes by dn/dt = -M (f'(n) - kappa lap n) with f(n) = n^2 (1-n)^2, so f'(n) = 4 n (n-1)(n-1/2).
// Initial condition: `n_grains` seeded circular grains with tanh profiles of width 2, summed and
// capped at 1; centres uniform in the domain, radii uniform in [5, 15], drawn from the
// parameter file's random seed. Post-processing: |grad n| and the free-energy density.
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
  set_initial_condition(const unsigned int       &index,
                        [[maybe_unused]] const unsigned int &component,
                        const dealii::Point<dim> &point,
                        number                   &scalar_value,
                        [[maybe_unused]] number  &vector_component_value) const override
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
        const ScalarValue f_bulk = n * n * n * n - 2.0 * n * n * n + n * n;
        variable_list.set_value_term(1, grad_n.norm());
        variable_list.set_value_term(2, f_bulk + 0.5 * kappa * grad_n.norm_square());
      }
  }

  number mobility;
  number kappa;
  std::vector<dealii::Point<dim>> centres;
  std::vector<double>             radii;
};

PRISMS_PF_END_NAMESPACE
