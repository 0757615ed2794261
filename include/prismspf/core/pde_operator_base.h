// Base class of a user's PDE operator (reference: include/prismspf/core/pde_operator_base.h:
// 46-165): initial and Dirichlet values on the host, the residual (compute_rhs) and the
// linear-operator (compute_lhs) callbacks evaluated at every quadrature point on the GPU.
//
// A CustomPDE written for the reference compiles against this header unchanged when the
// application is built with nvcc:
//   * compute_rhs / compute_lhs are `__host__ __device__` here, and the two macros at the
//     end of this file give the user's overrides the same execution space;
//   * the reference applications declare the overrides private; the macros also make them
//     public, so the cell kernel can call the final overrider directly (a qualified,
//     non-virtual call on the operator's bytes) instead of through a device vtable. An
//     empty, never-defined member declared just before each override carries the
//     declaration's leading `void`. Override declarations written `void compute_rhs(...)`
//     (the form the reference's applications use) are what the macros expect.
// The engine reads the operator object as plain bytes: its data members travel to the GPU
// as a kernel argument, and host-side members (the user-input pointers below, random-number
// distributions) are never touched there.
#pragma once

#include <prismspf/config.h>
#include <prismspf/core/field_container.h>
#include <prismspf/core/phase_field_tools.h>
#include <prismspf/core/simulation_timer.h>
#include <prismspf/core/types.h>
#include <prismspf/user_inputs/user_input_parameters.h>

#ifdef __CUDACC__
#define PPF_CALLBACK_SPACE __host__ __device__
// A GPU callback that calls a host-only function would have no device code to run: make
// that a compile-time error instead of nvcc's default warning.
#pragma nv_diag_error 20011
#pragma nv_diag_error 20014
#else
#define PPF_CALLBACK_SPACE
#endif

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim, unsigned int degree, typename number>
class SolveContext;

template <unsigned int dim, unsigned int degree, typename number>
class PDEOperatorBase {
 public:
  using SizeType = dealii::VectorizedArray<number>;

  explicit PDEOperatorBase(const UserInputParameters<dim>& _user_inputs, const PhaseFieldTools<dim>& _pf_tools)
      : user_inputs(&_user_inputs), pf_tools(&_pf_tools) {}

  PPF_CALLBACK_SPACE virtual ~PDEOperatorBase() {}

  // nodal initial value of field `index` (component `component` of a vector field)
  virtual void set_initial_condition([[maybe_unused]] const unsigned int& index,
                                     [[maybe_unused]] const unsigned int& component,
                                     [[maybe_unused]] const dealii::Point<dim>& point,
                                     [[maybe_unused]] number& scalar_value,
                                     [[maybe_unused]] number& vector_component_value) const {}

  // Dirichlet value on boundary `boundary_id`; defaults to the initial condition
  virtual void set_dirichlet(const unsigned int& index, [[maybe_unused]] const unsigned int& boundary_id,
                             const unsigned int& component, const dealii::Point<dim>& point,
                             [[maybe_unused]] const SimulationTimer& sim_timer, number& scalar_value,
                             number& vector_component_value) const {
    this->set_initial_condition(index, component, point, scalar_value, vector_component_value);
  }

  PPF_CALLBACK_SPACE virtual void compute_rhs([[maybe_unused]] FieldContainer<dim, degree, number>& variable_list,
                                              [[maybe_unused]] const SimulationTimer& sim_timer,
                                              [[maybe_unused]] unsigned int solver_id) const {}

  PPF_CALLBACK_SPACE virtual void compute_lhs([[maybe_unused]] FieldContainer<dim, degree, number>& variable_list,
                                              [[maybe_unused]] const SimulationTimer& sim_timer,
                                              [[maybe_unused]] unsigned int solver_id) const {}

  virtual void pre_solve_block([[maybe_unused]] SolveContext<dim, degree, number>& solve_context,
                               [[maybe_unused]] unsigned int solver_id) {}

  virtual void post_solve_block([[maybe_unused]] SolveContext<dim, degree, number>& solve_context,
                                [[maybe_unused]] unsigned int solver_id) {}

  [[nodiscard]] const UserInputParameters<dim>& get_user_inputs() const { return *user_inputs; }
  [[nodiscard]] const PhaseFieldTools<dim>& get_pf_tools() const { return *pf_tools; }

  void set_user_stop(bool flag) { user_stop = flag; }
  bool get_user_stop() { return user_stop; }

 private:
  const UserInputParameters<dim>* user_inputs = nullptr;
  const PhaseFieldTools<dim>* pf_tools = nullptr;
  bool user_stop = false;
};

PRISMS_PF_END_NAMESPACE

// the user's `void compute_rhs(...) const override` becomes a public __host__ __device__
// override (see the header comment)
#define compute_rhs ppf_compute_rhs_declared_(); public: PPF_CALLBACK_SPACE void compute_rhs
#define compute_lhs ppf_compute_lhs_declared_(); public: PPF_CALLBACK_SPACE void compute_lhs
// the user's `void pre_solve_block(...) override` / `void post_solve_block(...) override`
// become public host overrides, so Problem can tell whether the operator declares them (an
// operator without hooks keeps the CUDA-graph increment loop)
#define pre_solve_block ppf_pre_solve_block_declared_(); public: void pre_solve_block
#define post_solve_block ppf_post_solve_block_declared_(); public: void post_solve_block
