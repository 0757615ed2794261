// SolveContext handed to a user's pre_solve_block / post_solve_block hooks (reference:
// include/prismspf/solvers/solve_context.h:31-214, the hooks at
// include/prismspf/core/pde_operator_base.h:96-108, called around every solved block by
// Problem::solve_increment, src/core/problem.cc:436-451).
//
// The reference context exposes its deal.II managers (triangulation, DoF handlers, constraints,
// matrix-free objects, solution vectors). This engine keeps that state on the GPU behind its C
// ABI, so the context offers what a hook can use here: the field attributes, the user inputs,
// the simulation timer of the increment being solved, the operator itself (set_user_stop), the
// engine handle, and host copies of solution vectors in the engine's node order. A hook that
// reaches for a deal.II manager does not compile.
#pragma once

#include <vector>

#include <ppf_gb300.h>
#include <prismspf/config.h>
#include <prismspf/core/field_attributes.h>
#include <prismspf/core/simulation_timer.h>
#include <prismspf/user_inputs/user_input_parameters.h>

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim, unsigned int degree, typename number>
class PDEOperatorBase;

template <unsigned int dim, unsigned int degree, typename number>
class SolveContext {
 public:
  SolveContext(const std::vector<FieldAttributes>& fields, const UserInputParameters<dim>& inputs,
               PDEOperatorBase<dim, degree, number>& pde, ppf_handle h)
      : field_attributes(&fields), user_inputs(&inputs), pde_operator(&pde), handle(h) {}

  [[nodiscard]] const std::vector<FieldAttributes>& get_field_attributes() const { return *field_attributes; }
  [[nodiscard]] const UserInputParameters<dim>& get_user_inputs() const { return *user_inputs; }
  [[nodiscard]] const SimulationTimer& get_simulation_timer() const { return timer; }
  [[nodiscard]] SimulationTimer& get_simulation_timer() { return timer; }
  [[nodiscard]] const PDEOperatorBase<dim, degree, number>& get_pde_operator() const { return *pde_operator; }
  [[nodiscard]] PDEOperatorBase<dim, degree, number>& get_pde_operator() { return *pde_operator; }

  // the engine handle (ppf_gb300.h), for hooks that call the C ABI themselves
  [[nodiscard]] ppf_handle get_handle() const { return handle; }

  // host copy of field `index` at `age` (0 current, 1.. old), engine node order (the lattice,
  // component-major for vector fields; the DoF list on adaptive meshes)
  [[nodiscard]] std::vector<double> get_solution(unsigned int index, unsigned int age = 0) const {
    std::vector<double> v((size_t)ppf_field_length(handle, (int)index));
    if (ppf_download_state(handle, (int)index, (int)age, v.data(), PPF_ORDER_NATIVE) != PPF_OK) v.clear();
    return v;
  }

  // the increment's timer, set by the driver before each hook
  void set_simulation_timer(const SimulationTimer& t) { timer = t; }

 private:
  const std::vector<FieldAttributes>* field_attributes;
  const UserInputParameters<dim>* user_inputs;
  PDEOperatorBase<dim, degree, number>* pde_operator;
  ppf_handle handle;
  SimulationTimer timer;
};

PRISMS_PF_END_NAMESPACE
