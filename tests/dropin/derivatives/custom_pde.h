// Test application: the FieldContainer getters the applications under examples/ do not use
// (Hessian, Hessian diagonal, Laplacian, divergence, curl, symmetric gradient, quadrature-point
// location, element volume), written into post-processed fields. The inputs are quadratic
// polynomials, which FE_Q(2) represents exactly, so every output has a closed form:
//   u = 1 + x + 2y + x^2/2 + 3xy + 5y^2/2    (u_xx = 1, u_xy = 3, u_yy = 5, lap u = 6)
//   w = (x^2 + y, x y)                       (div w = 3x, curl w = y - 1, sym(grad w)_xy = (1 + y)/2)
#include <prismspf/core/pde_operator_base.h>

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim, unsigned int degree, typename number>
class CustomPDE : public PDEOperatorBase<dim, degree, number>
{
public:
  using ScalarValue = dealii::VectorizedArray<number>;

  CustomPDE(const UserInputParameters<dim> &_user_inputs, PhaseFieldTools<dim> &_pf_tools)
    : PDEOperatorBase<dim, degree, number>(_user_inputs, _pf_tools)
  {}

private:
  void
  set_initial_condition(const unsigned int       &index,
                        const unsigned int       &component,
                        const dealii::Point<dim> &p,
                        number                   &scalar_value,
                        number                   &vector_component_value) const override
  {
    const double x = p[0], y = p[1];
    if (index == 0)
      scalar_value = 1.0 + x + 2.0 * y + 0.5 * x * x + 3.0 * x * y + 2.5 * y * y;
    else if (index == 1)
      vector_component_value = component == 0 ? x * x + y : x * y;
  }

  void
  compute_rhs(FieldContainer<dim, degree, number> &variable_list,
              [[maybe_unused]] const SimulationTimer &sim_timer,
              unsigned int                         solve_block_id) const override
  {
    if (solve_block_id == 2)
      {
        // hess_u packs three entries with distinct weights: u_xx + 10 u_yx + 100 u_yy = 531
        const auto        hess  = variable_list.template get_hessian<Scalar, Current>(0);
        const auto        hdiag = variable_list.template get_hessian_diagonal<Scalar, Current>(0);
        const ScalarValue lap   = variable_list.template get_laplacian<Scalar, Current>(0);
        const ScalarValue div   = variable_list.template get_divergence<Vector, Current>(1);
        variable_list.set_value_term(2, lap);
        variable_list.set_value_term(3, hess[0][0] + 10.0 * hess[1][0] + 100.0 * hdiag[1]);
        variable_list.set_value_term(4, div);
      }
    else if (solve_block_id == 3)
      {
        const auto curl = variable_list.template get_curl<Vector, Current>(1);
        const auto sym  = variable_list.template get_symmetric_gradient<Vector, Current>(1);
        const auto x    = variable_list.get_q_point_location();
        variable_list.set_value_term(5, curl[0]);
        variable_list.set_value_term(6, sym[0][1]);
        variable_list.set_value_term(7, x[0] + variable_list.get_element_volume());
      }
  }
};

PRISMS_PF_END_NAMESPACE
