// Linear elasticity with the eigenstrain of seeded spherical inclusions (the 3-D elasticity
// benchmark configuration): div(C : (eps(u) - eps*)) = 0 with eps* = e0 * min(1, sum_i h_i) I,
// h_i = (1 - tanh((|x - x_i| - r_i) / w)) / 2, and u = 0 on the x = 0 face (boundary id 0).
// The inclusions are Model constants (inclusion_<i> = (x, y, z), radius_<i>) so that a
// driver can place them; they are stored in the operator object itself because the
// callbacks run on the GPU, where only the object's own bytes are available.
#include <prismspf/core/pde_operator_base.h>
#include <prismspf/utilities/mechanics.h>

#include <string>

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim, unsigned int degree, typename number>
class CustomPDE : public PDEOperatorBase<dim, degree, number>
{
public:
  using ScalarValue = dealii::VectorizedArray<number>;
  using VectorGrad  = dealii::Tensor<2, dim, ScalarValue>;
  using PDEOperatorBase<dim, degree, number>::get_user_inputs;

  static constexpr unsigned int max_inclusions = 64;

  CustomPDE(const UserInputParameters<dim> &_user_inputs, PhaseFieldTools<dim> &_pf_tools)
    : PDEOperatorBase<dim, degree, number>(_user_inputs, _pf_tools)
    , stiffness(get_user_inputs().user_constants.get_elasticity_tensor("stiffness"))
    , eigenstrain(get_user_inputs().user_constants.get_double("eigenstrain"))
    , width(get_user_inputs().user_constants.get_double("interface_width"))
    , n_inclusions(get_user_inputs().user_constants.get_int("n_inclusions"))
  {
    if (n_inclusions > (int) max_inclusions)
      throw std::invalid_argument("too many inclusions");
    for (int i = 0; i < n_inclusions; ++i)
      {
        const auto c = get_user_inputs().user_constants.get_rank_1_tensor("inclusion_" + std::to_string(i));
        for (unsigned int d = 0; d < dim; ++d)
          inclusions[i][d] = c[d];
        inclusions[i][3] = get_user_inputs().user_constants.get_double("radius_" + std::to_string(i));
      }
  }

private:
  void
  set_dirichlet([[maybe_unused]] const unsigned int       &index,
                [[maybe_unused]] const unsigned int       &boundary_id,
                [[maybe_unused]] const unsigned int       &component,
                [[maybe_unused]] const dealii::Point<dim> &point,
                [[maybe_unused]] const SimulationTimer    &sim_timer,
                number                                    &scalar_value,
                number                                    &vector_component_value) const override
  {
    scalar_value           = 0.0;
    vector_component_value = 0.0;
  }

  void
  compute_rhs(FieldContainer<dim, degree, number> &variable_list,
              [[maybe_unused]] const SimulationTimer &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    if (solve_block_id == 1)
      {
        const dealii::Point<dim, ScalarValue> x = variable_list.get_q_point_location();
        ScalarValue                           h(0.0);
        for (int i = 0; i < n_inclusions; ++i)
          {
            ScalarValue r2(0.0);
            for (unsigned int d = 0; d < dim; ++d)
              r2 += (x[d] - inclusions[i][d]) * (x[d] - inclusions[i][d]);
            h += 0.5 * (1.0 - std::tanh((std::sqrt(r2) - inclusions[i][3]) / width));
          }
        VectorGrad eps_star;
        for (unsigned int d = 0; d < dim; ++d)
          eps_star[d][d] = eigenstrain * std::min(h, ScalarValue(1.0));
        VectorGrad stress;
        Mechanics::compute_stress<dim, ScalarValue>(stiffness, eps_star, stress);
        variable_list.set_gradient_term(0, -stress);
      }
  }

  void
  compute_lhs(FieldContainer<dim, degree, number> &variable_list,
              [[maybe_unused]] const SimulationTimer &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    if (solve_block_id == 1)
      {
        const VectorGrad strain = variable_list.template get_symmetric_gradient<Vector, LHS>(0);
        VectorGrad       stress;
        Mechanics::compute_stress<dim, ScalarValue>(stiffness, strain, stress);
        variable_list.set_gradient_term(0, stress);
      }
  }

  dealii::Tensor<2, Mechanics::voigt_tensor_size<dim>, number> stiffness;
  number                                                        eigenstrain;
  number                                                        width;
  int                                                           n_inclusions;
  number inclusions[max_inclusions][4] = {};
};

PRISMS_PF_END_NAMESPACE
