// Drop-in Problem (reference: include/prismspf/core/problem.h, src/core/problem.cc:31-557):
// builds the system from the fields, solve blocks, parameter file and the user's operator,
// and runs the increment loop on the GPU through the engine's C ABI (ppf_gb300.h).
//
//   Problem<dim, degree, double> problem(fields, solve_blocks, user_inputs, pf_tools, pde);
//   problem.solve();
//
// Build the application with nvcc (`-x cu`): the constructor instantiates the matrix-free
// cell kernel for the user's CustomPDE in the application's own translation unit and hands
// the engine a launcher for it (ppf_create_custom). Host-side parts follow the reference:
//   * initial conditions: set_initial_condition at every support point of every cell, cells
//     in deal.II's order, points in FE_Q's order, for the fields of Primary blocks
//     (SolverBase::set_initial_condition, solver_base.h:178-229 with
//     InitialCondition::vector_value, initial_conditions.cc:35-62);
//   * Dirichlet values: set_dirichlet at the constrained boundary nodes, re-evaluated before
//     every increment when the parameter file marks them time dependent;
//   * linear-solver parameters from "linear solver parameters: k" by solve-block id
//     (problem.cc:178-200);
//   * output increments from the "output" subsection: VTU (or a one-piece PVTU) of every
//     field and the reference's log lines (field l2-norm and integrated value,
//     problem.cc:505-552);
//   * a non-finite solution writes the output of that increment and throws ExcNaN;
//   * "mesh adaptivity = true": the engine's adaptive mesh (ppf_set_adaptivity) with the
//     parameter file's min/max refinement, remeshing period and refinement criteria, for
//     degrees 1 and 2 (other degrees run on the uniform mesh with a note; Linear and Newton
//     blocks without a preconditioner); the initial condition is set on the initial uniform
//     mesh and carried through the refinement passes as the reference's solution transfer does,
//     Dirichlet values come from set_dirichlet at the nodes of every mesh, and the output
//     writes the active cells of the current mesh.
//   * an operator that declares pre_solve_block / post_solve_block gets them called around
//     every block solved in an increment with a SolveContext (prismspf/solvers/solve_context.h),
//     the increment loop then running block by block (ppf_increment_block); set_user_stop(true)
//     in a hook ends the run after that increment with its output written and "Exit triggered
//     by user!" (problem.cc:436-477, 392-414);
//   * NucleationRate blocks run on output increments and on increments divisible by the
//     `nucleation period` (nucleation_parameters.cc:110-113).
// Not carried over: stochastic nucleation, checkpoints, initial conditions from files. Newton
// blocks run with cg or bicgstab (no preconditioner, or Chebyshev for single-field blocks).
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include <ppf_gb300.h>
#include <prismspf/config.h>
#include <prismspf/core/dependencies.h>
#include <prismspf/core/field_attributes.h>
#include <prismspf/core/pde_operator_base.h>
#include <prismspf/core/phase_field_tools.h>
#include <prismspf/core/simulation_timer.h>
#include <prismspf/core/solution_output.h>
#include <prismspf/core/solve_block.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/solvers/solve_context.h>
#include <prismspf/user_inputs/user_input_parameters.h>

// the hook names are rewritten for user classes by pde_operator_base.h; this header calls them
#pragma push_macro("pre_solve_block")
#pragma push_macro("post_solve_block")
#undef pre_solve_block
#undef post_solve_block

#ifdef __CUDACC__
#include <prismspf/gpu/launch.cuh>
#endif

#pragma push_macro("compute_rhs")
#pragma push_macro("compute_lhs")
#undef compute_rhs
#undef compute_lhs

PRISMS_PF_BEGIN_NAMESPACE

class ExcNaN : public std::runtime_error {
 public:
  explicit ExcNaN(const std::string& m) : std::runtime_error("ExcNaN: " + m) {}
};

class ExcEngine : public std::runtime_error {
 public:
  ExcEngine(int code, const std::string& m) : std::runtime_error(m), status(code) {}
  int status;
};

namespace detail {

// The user's operator as the cell kernel sees it: the object's bytes, with the callbacks
// forwarded to the final overriders by qualified (non-virtual) calls.
template <class PDE>
struct UserOperator {
  alignas(alignof(PDE)) unsigned char bytes[sizeof(PDE)];

  template <unsigned int dim, unsigned int degree, typename number>
  PPF_CALLBACK_SPACE void compute_rhs(FieldContainer<dim, degree, number>& fc, const SimulationTimer& t,
                                      unsigned int id) const {
    reinterpret_cast<const PDE*>(bytes)->PDE::compute_rhs(fc, t, id);
  }
  template <unsigned int dim, unsigned int degree, typename number>
  PPF_CALLBACK_SPACE void compute_lhs(FieldContainer<dim, degree, number>& fc, const SimulationTimer& t,
                                      unsigned int id) const {
    reinterpret_cast<const PDE*>(bytes)->PDE::compute_lhs(fc, t, id);
  }
};

// true when PDE itself declares pre_solve_block or post_solve_block
template <class PDE, unsigned int dim, unsigned int degree, typename number>
constexpr bool declares_hooks() {
  using Own = void (PDE::*)(SolveContext<dim, degree, number>&, unsigned int);
  return std::is_same_v<decltype(&PDE::pre_solve_block), Own> ||
         std::is_same_v<decltype(&PDE::post_solve_block), Own>;
}

// true when PDE itself declares compute_lhs (a Linear block needs it)
template <class PDE, unsigned int dim, unsigned int degree, typename number>
constexpr bool declares_lhs() {
  using Own = void (PDE::*)(FieldContainer<dim, degree, number>&, const SimulationTimer&, unsigned int) const;
  return std::is_same_v<decltype(&PDE::compute_lhs), Own>;
}

#ifdef __CUDACC__
template <class PDE, int dim, int degree, bool lhs>
int launch_user_operator(int d, int k, int mode, int precision, const void* cell_launch, const void* object,
                         size_t smem, void* stream) {
  if (d != dim || k != degree || precision != 0) return (int)cudaErrorInvalidValue;
  const ppf::CellLaunch& P = *static_cast<const ppf::CellLaunch*>(cell_launch);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  using Op = UserOperator<PDE>;
  if (mode == ppf::MODE_RHS) return (int)ppf::launch_cell_kernel<Op, dim, degree, ppf::MODE_RHS, double>(P, object, smem, s);
  // adaptive meshes: the launch record is an AmrCellLaunch
  if (mode == (ppf::MODE_RHS | ppf::MODE_AMR))
    return (int)ppf::launch_amr_operator<Op, dim, degree, ppf::MODE_RHS>(cell_launch, object, smem, s);
  if constexpr (lhs) {
    if (mode == (ppf::MODE_LHS | ppf::MODE_AMR))
      return (int)ppf::launch_amr_operator<Op, dim, degree, ppf::MODE_LHS>(cell_launch, object, smem, s);
    if (mode == ppf::MODE_LHS)
      return (int)ppf::launch_cell_kernel<Op, dim, degree, ppf::MODE_LHS, double>(P, object, smem, s);
    if (mode == ppf::MODE_DIAG)
      return (int)ppf::launch_cell_kernel<Op, dim, degree, ppf::MODE_DIAG, double>(P, object, smem, s);
  }
  return (int)cudaErrorInvalidValue;
}
#endif

inline unsigned char age_flags(const Dependency& d, int age) {
  if (age == 0) return (unsigned char)d.flag;
  if (age == 5) return (unsigned char)d.src_flag;
  return age - 1 < (int)d.old_flags.size() ? (unsigned char)d.old_flags[age - 1] : 0;
}

}  // namespace detail

template <unsigned int dim, unsigned int degree, typename number>
class Problem {
 public:
  using Base = PDEOperatorBase<dim, degree, number>;

  template <class PDE>
  Problem(const std::vector<FieldAttributes>& _field_attributes, const std::vector<SolveBlock>& _solve_blocks,
          const UserInputParameters<dim>& _user_inputs, PhaseFieldTools<dim>& _pf_tools, PDE& _pde_operator)
      : field_attributes(_field_attributes),
        solve_blocks(_solve_blocks),
        user_inputs(&_user_inputs),
        pf_tools(&_pf_tools),
        pde(&_pde_operator) {
    static_assert(std::is_base_of_v<Base, PDE>, "the operator must derive from PDEOperatorBase<dim, degree, number>");
    static_assert(std::is_same_v<number, double>, "the GPU engine computes the drop-in path in FP64 (number = double)");
    const unsigned char* b = reinterpret_cast<const unsigned char*>(&_pde_operator);
    object_source = b;
    object_size = sizeof(PDE);
    has_lhs = detail::declares_lhs<PDE, dim, degree, number>();
    has_hooks = detail::declares_hooks<PDE, dim, degree, number>();
    hooks = &_pde_operator;
#ifdef __CUDACC__
    launcher = &detail::launch_user_operator<PDE, (int)dim, (int)degree,
                                             detail::declares_lhs<PDE, dim, degree, number>()>;
#endif
    // linear / nonlinear solver parameters by solve-block id (problem.cc:178-200)
    for (auto& sb : solve_blocks) {
      auto it = user_inputs->linear_solve_parameters.linear_solvers.find((unsigned)sb.id);
      if (it != user_inputs->linear_solve_parameters.linear_solvers.end()) sb.linear_solver_parameters = it->second;
      auto nt = user_inputs->nonlinear_solve_parameters.nonlinear_solvers.find((unsigned)sb.id);
      if (nt != user_inputs->nonlinear_solve_parameters.nonlinear_solvers.end())
        sb.nonlinear_solver_parameters = nt->second;
    }
  }

  Problem(const Problem&) = delete;
  Problem& operator=(const Problem&) = delete;
  ~Problem() {
    if (handle) ppf_destroy(handle);
  }

  void solve() {
    init_system();
    if (has_hooks) {
      solve_with_hooks();
      return;
    }
    const TemporalDiscretization& time = user_inputs->temporal_discretization;
    const unsigned int n = time.n_increments;
    std::vector<unsigned int> outputs;
    for (unsigned int o : user_inputs->output_parameters.output_list)
      if (o <= n) outputs.push_back(o);
    unsigned int next = 0;  // next increment to run
    auto run_to = [&](unsigned int last, int output_every) {
      while (next <= last) {
        const unsigned int stop = time_dependent ? next : last;
        if (time_dependent) update_dirichlet(next);
        const int rc = ppf_run(handle, stop, output_every);
        if (rc == PPF_ERR_NAN) {
          next = current_increment();
          write_output(next == 0 ? 0 : next - 1);
          throw ExcNaN("Exiting early.");
        }
        check(rc, "increment loop");
        next = stop + 1;
      }
    };
    for (unsigned int o : outputs) {
      if (o > 0) run_to(o - 1, 0);
      run_to(o, o == 0 ? 1 : (int)o);
      write_output(o);
    }
    run_to(n, 0);
    check(ppf_synchronize(handle), "synchronize");
  }

  // engine handle (valid after solve() has started)
  ppf_handle get_handle() const { return handle; }

 private:
  // Problem::solve with the operator's pre/post_solve_block hooks (problem.cc:416-557): the
  // blocks of an increment one at a time, each solved block between its two hooks, then the
  // remeshing step, the rotation, the output, and the user stop (exit status 3).
  void solve_with_hooks() {
    const unsigned int n = user_inputs->temporal_discretization.n_increments;
    std::set<unsigned int> outputs;
    for (unsigned int o : user_inputs->output_parameters.output_list)
      if (o <= n) outputs.insert(o);
    SolveContext<dim, degree, number> ctx(field_attributes, *user_inputs, *hooks, handle);
    for (unsigned int inc = current_increment(); inc <= n; ++inc) {
      if (time_dependent) update_dirichlet(inc);
      const bool is_output = outputs.count(inc) != 0;
      const bool attempt = user_inputs->nucleation_parameters.should_attempt_nucleation(inc);
      for (size_t b = 0; b < solve_blocks.size(); ++b) {
        const SolveTiming t = solve_blocks[b].solve_timing;
        const bool due = !(t == PostProcess && !is_output) && !(t == NucleationRate && !(is_output || attempt));
        if (due) {
          double time = 0.0;
          unsigned int cur = 0;
          ppf_get_time(handle, &cur, &time);
          SimulationTimer timer(user_inputs->temporal_discretization.dt, 0.0);
          timer.set_increment(cur);
          timer.set_time(time);
          ctx.set_simulation_timer(timer);
          hooks->pre_solve_block(ctx, (unsigned int)solve_blocks[b].id);
        }
        const int rc = ppf_increment_block(handle, (int)b, is_output ? 1 : 0);
        if (rc != PPF_OK && rc != PPF_ERR_NOCONV) check(rc, "solve block");
        if (due) hooks->post_solve_block(ctx, (unsigned int)solve_blocks[b].id);
      }
      if (adaptive) check(ppf_remesh_if_due(handle), "remeshing");
      const int rc = ppf_end_increment(handle);
      if (rc == PPF_ERR_NAN) {
        write_output(inc);
        throw ExcNaN("Exiting early.");
      }
      check(rc, "end of increment");
      const bool stop = hooks->get_user_stop();
      if (is_output || stop) write_output(inc);
      if (stop) {
        std::cout << "Exit triggered by user!" << std::endl;
        break;
      }
    }
    check(ppf_synchronize(handle), "synchronize");
  }

 public:

 private:
  void check(int rc, const char* what) const {
    if (rc != PPF_OK) {
      const char* m = ppf_last_error(handle);
      throw ExcEngine(rc, std::string(what) + ": " + (m && *m ? m : "engine error ") + " (status " + std::to_string(rc) + ")");
    }
  }

  unsigned int current_increment() const {
    unsigned int inc = 0;
    double t = 0.0;
    ppf_get_time(handle, &inc, &t);
    return inc;
  }

  void init_system() {
    if (handle) return;
    const auto& sd = user_inputs->spatial_discretization;
    const auto& mesh = sd.rectangular_mesh;
    // adaptive meshes (refinement_manager.cc) for degrees 1 and 2; other configurations run on
    // the uniform mesh with a note. Linear and Newton blocks solve without a preconditioner there
    // (problem.cc:356-359 refuses multigrid with adaptivity).
    adaptive = false;
    if (sd.has_adaptivity) {
      for (const auto& sb : solve_blocks)
        if ((sb.solve_type == SolveType::Linear || sb.solve_type == SolveType::Newton) &&
            sb.linear_solver_parameters.preconditioner != PreconditionerType::None)
          throw std::invalid_argument("AMR cannot be enabled when using multigrid preconditioners currently.");
      std::string why;
      if (dim < 2) why = "one-dimensional meshes";
      else if (degree > 2) why = "degree > 2";
      if (why.empty()) {
        if (sd.max_refinement < sd.global_refinement)
          throw std::invalid_argument("The maximum refinement level must be greater than or equal to the global refinement level.");
        if (sd.min_refinement > sd.global_refinement)
          throw std::invalid_argument("The minimum refinement level must be less than or equal to the global refinement level.");
        adaptive = true;
      } else {
        std::cout << "note: mesh adaptivity is not applied with " << why << "; running on the uniform mesh (global refinement "
                  << sd.global_refinement << ")" << std::endl;
      }
    }
    for (const auto& s : user_inputs->not_applied) std::cout << "note: not applied: " << s << std::endl;
    if (field_attributes.empty() || field_attributes.size() > PPF_MAX_FIELDS)
      throw std::invalid_argument("between 1 and 8 fields are supported");
    if (solve_blocks.size() > PPF_MAX_BLOCKS) throw std::invalid_argument("at most 8 solve blocks are supported");

    ppf_mesh_desc m{};
    m.dim = (int)dim;
    m.degree = (int)degree;
    m.global_refinement = (int)sd.global_refinement;
    for (unsigned int d = 0; d < dim; ++d) {
      m.subdivisions[d] = (int)mesh.subdivisions[d];
      m.lower[d] = mesh.lower_bound[d];
      m.size[d] = mesh.size[d] - mesh.lower_bound[d];
      m.periodic[d] = mesh.periodic_directions.count(d) ? 1 : 0;
    }
    for (unsigned int d = dim; d < 3; ++d) {
      m.subdivisions[d] = 1;
      m.size[d] = 1.0;
    }
    lattice.dim = (int)dim;
    lattice.degree = (int)degree;
    lattice.N = 1;
    for (unsigned int d = 0; d < 3; ++d) {
      lattice.nc[d] = d < dim ? m.subdivisions[d] << m.global_refinement : 1;
      lattice.nn[d] = d < dim ? (int)degree * lattice.nc[d] + 1 : 1;
      lattice.lower[d] = d < dim ? m.lower[d] : 0.0;
      lattice.h[d] = d < dim ? m.size[d] / lattice.nc[d] : 1.0;
      lattice.N *= lattice.nn[d];
    }

    // fields and their boundary conditions (constraint_manager.cc:143-304)
    std::vector<ppf_field_desc> fd(field_attributes.size());
    dirichlet_fields.assign(field_attributes.size(), false);
    time_dependent = false;
    for (size_t f = 0; f < field_attributes.size(); ++f) {
      std::memset(&fd[f], 0, sizeof(ppf_field_desc));
      fd[f].rank = field_attributes[f].field_type == TensorRank::Vector ? 1 : 0;
      auto it = user_inputs->boundary_parameters.boundary_condition_list.find(field_attributes[f].name);
      if (it == user_inputs->boundary_parameters.boundary_condition_list.end()) continue;
      const int ncomp = fd[f].rank ? (int)dim : 1;
      for (const auto& [comp, conds] : it->second.component_constraints) {
        if ((int)comp >= ncomp) continue;
        for (const auto& [bid, cond] : conds) {
          if (bid >= 2 * dim) continue;
          if (cond == Condition::Dirichlet) {
            fd[f].dirichlet[comp][bid] = 1;
            dirichlet_fields[f] = true;
          } else if (cond == Condition::Periodic) {
            if (!mesh.periodic_directions.count(bid / 2))
              throw std::invalid_argument("field " + field_attributes[f].name +
                                          ": Periodic boundary condition on a direction the mesh is not periodic in");
          } else if (cond == Condition::Neumann) {
            throw std::invalid_argument("Neumann boundary conditions are not supported by this engine");
          }
        }
      }
      if (dirichlet_fields[f] && it->second.time_dependent) time_dependent = true;
    }

    // solve blocks (solve_block.h:56-127)
    std::vector<ppf_block_desc> bd(solve_blocks.size());
    bool any_linear = false;
    for (size_t b = 0; b < solve_blocks.size(); ++b) {
      const SolveBlock& sb = solve_blocks[b];
      sb.validate();
      std::memset(&bd[b], 0, sizeof(ppf_block_desc));
      bd[b].id = sb.id;
      bd[b].solve_type = (int)sb.solve_type;
      bd[b].solve_timing = (int)sb.solve_timing;
      bd[b].n_fields = (int)sb.field_indices.size();
      int i = 0;
      for (unsigned int f : sb.field_indices) bd[b].field_indices[i++] = (int)f;
      for (const auto* deps : {&sb.dependencies_rhs, &sb.dependencies_lhs})
        for (const auto& [f, d] : *deps) {
          if (f >= field_attributes.size()) throw std::invalid_argument("dependency on an unknown field index");
          if (d.old_flags.size() > 4)
            for (size_t a = 4; a < d.old_flags.size(); ++a)
              if (d.old_flags[a] != EvalFlags::nothing)
                throw std::invalid_argument("dependencies older than old_4 are not supported");
          for (int age = 0; age < PPF_NAGE; ++age)
            (deps == &sb.dependencies_rhs ? bd[b].dep_rhs : bd[b].dep_lhs)[f][age] = detail::age_flags(d, age);
        }
      any_linear |= sb.solve_type == SolveType::Linear || sb.solve_type == SolveType::Newton;
    }
    if (any_linear && !has_lhs)
      throw std::invalid_argument("a Linear or Newton solve block needs compute_lhs in the operator");

    const SimulationTimer t0(user_inputs->temporal_discretization.dt, user_inputs->temporal_discretization.initial_time);
    ppf_model_desc md{};
    md.name = "custom_pde";
    md.has_lhs = has_lhs ? 1 : 0;
    md.object = object_source;
    md.object_size = object_size;
#ifdef __CUDACC__
    md.launch = launcher;
    md.cell_launch_size = sizeof(ppf::CellLaunch);
#else
    throw std::runtime_error("build the application with nvcc (-x cu) so the operator's GPU kernel is compiled");
#endif
    check(ppf_create_custom(&m, fd.data(), (int)fd.size(), bd.data(), (int)bd.size(), &md, t0.get_timestep(), &handle),
          "set-up");
    if (user_inputs->temporal_discretization.initial_time != 0.0)
      check(ppf_set_time(handle, 0, user_inputs->temporal_discretization.initial_time), "start time");
    check(ppf_set_nucleation_period(handle, user_inputs->nucleation_parameters.nucleation_period),
          "nucleation period");
    if (adaptive) {
      ppf_adaptivity a{};
      a.min_refinement = (int)sd.min_refinement;
      a.max_refinement = (int)sd.max_refinement;
      // remeshing period: increments between passes (the default UINT_MAX: only increment 0)
      a.remeshing_period = sd.remeshing_period > (unsigned)INT32_MAX ? 0 : (int)sd.remeshing_period;
      for (const auto& [name, c] : sd.refinement_criteria) {
        if (c.criterion == RefinementFlags::Nothing) continue;
        int f = -1;
        for (size_t i = 0; i < field_attributes.size(); ++i)
          if (field_attributes[i].name == name) f = (int)i;
        if (f < 0) throw std::invalid_argument("refinement criterion for an unknown field " + name);
        if (a.n_criteria >= PPF_MAX_FIELDS) throw std::invalid_argument("too many refinement criteria");
        a.criterion_field[a.n_criteria] = f;
        a.criterion_flags[a.n_criteria] = (int)c.criterion;
        a.value_lower[a.n_criteria] = c.value_lower_bound;
        a.value_upper[a.n_criteria] = c.value_upper_bound;
        a.gradient_lower[a.n_criteria] = c.gradient_lower_bound;
        a.n_criteria++;
      }
      check(ppf_set_adaptivity(handle, &a), "mesh adaptivity");
    }

    // linear (and Newton) solver parameters (linear_solver.h:220-402, newton_solver.h:73-156)
    for (size_t b = 0; b < solve_blocks.size(); ++b) {
      const SolveType st = solve_blocks[b].solve_type;
      if (st != SolveType::Linear && st != SolveType::Newton) continue;
      const LinearSolverParameters& L = solve_blocks[b].linear_solver_parameters;
      ppf_linear_params p;
      ppf_default_linear_params(&p);
      if (L.solver_type == "cg") p.solver_type = 0;
      else if (L.solver_type == "bicgstab" && st == SolveType::Newton) p.solver_type = 1;
      else throw std::invalid_argument("linear solver type " + L.solver_type + " is not supported for this block");
      p.tolerance_type = (int)L.tolerance_type;
      p.tolerance = L.tolerance;
      p.max_iterations = (int)L.max_iterations;
      p.preconditioner = (int)L.preconditioner;
      p.mg_depth = (int)L.mg_depth;
      p.smoother_degree = (int)L.chebyshev_parameters.degree;
      p.smoothing_range = L.chebyshev_parameters.smoothing_range;
      p.eig_cg_iterations = (int)L.chebyshev_parameters.eig_cg_n_iterations;
      check(ppf_set_linear_params(handle, (int)b, &p), "linear solver parameters");
      if (st == SolveType::Newton) {
        const NonlinearSolverParameters& N = solve_blocks[b].nonlinear_solver_parameters;
        check(ppf_set_newton_params(handle, (int)b, (int)N.max_iterations, N.tolerance_value, N.step_length),
              "Newton solver parameters");
      }
    }

    update_dirichlet(0);
    apply_initial_conditions();
  }

  // node coordinates of the lattice (Gauss-Lobatto nodes inside each cell)
  dealii::Point<dim> node_point(long long node) const {
    static thread_local std::vector<double> gl;
    if ((int)gl.size() != (int)degree + 1) gl = output::gauss_lobatto_unit((int)degree);
    long long idx[3] = {node % lattice.nn[0], (node / lattice.nn[0]) % lattice.nn[1],
                        node / ((long long)lattice.nn[0] * lattice.nn[1])};
    dealii::Point<dim> p;
    for (unsigned int d = 0; d < dim; ++d) {
      const long long cell = std::min<long long>(idx[d] / degree, lattice.nc[d] - 1);
      const int a = (int)(idx[d] - cell * degree);
      p[d] = lattice.lower[d] + lattice.h[d] * ((double)cell + gl[a]);
    }
    return p;
  }

  // set_dirichlet at one boundary point, for the engine's Dirichlet nodes of adaptive meshes
  static double dirichlet_point(void* user, int field, int comp, int bid, const double* x, double time) {
    const Problem* self = static_cast<const Problem*>(user);
    const auto& T = self->user_inputs->temporal_discretization;
    SimulationTimer timer(T.dt, time);
    timer.set_increment(T.dt != 0.0 ? (unsigned int)std::llround((time - T.initial_time) / T.dt) : 0u);
    dealii::Point<dim> p;
    for (unsigned int d = 0; d < dim; ++d) p[d] = x[d];
    number s[3] = {0, 0, 0};
    if (self->field_attributes[(size_t)field].field_type != TensorRank::Vector) {
      self->pde->set_dirichlet((unsigned)field, (unsigned)bid, 0, p, timer, s[0], s[0]);
      return s[0];
    }
    self->pde->set_dirichlet((unsigned)field, (unsigned)bid, (unsigned)comp, p, timer, s[0], s[comp]);
    return s[comp];
  }

  void apply_initial_conditions() {
    std::set<unsigned int> ic_fields;
    for (const auto& sb : solve_blocks)
      if (sb.solve_timing == SolveTiming::Primary) ic_fields.insert(sb.field_indices.begin(), sb.field_indices.end());
    if (ic_fields.empty()) return;
    const long long ncells = ppf_n_cells(handle);
    const int ppc = (int)std::pow(degree + 1, dim);
    std::vector<std::vector<double>> vals(field_attributes.size());
    // lattice-order vectors of the initial mesh (adaptive meshes start from it too)
    for (unsigned int f : ic_fields)
      vals[f].assign((size_t)((field_attributes[f].field_type == TensorRank::Vector ? dim : 1) * lattice.N), 0.0);
    const long long chunk = 1 << 15;
    std::vector<long long> nodes;
    for (long long c0 = 0; c0 < ncells; c0 += chunk) {
      const long long nc = std::min(chunk, ncells - c0);
      nodes.resize((size_t)(nc * ppc));
      check(ppf_dealii_cell_nodes(handle, c0, nc, nodes.data()), "support points");
      for (long long i = 0; i < nc * ppc; ++i) {
        const long long node = nodes[(size_t)i];
        const dealii::Point<dim> p = node_point(node);
        for (unsigned int f : ic_fields) {
          // InitialCondition::vector_value: scalar_value aliases component 0
          number v[3] = {0, 0, 0};
          const bool vec = field_attributes[f].field_type == TensorRank::Vector;
          if (!vec) {
            pde->set_initial_condition(f, 0, p, v[0], v[0]);
            vals[f][(size_t)node] = v[0];
          } else {
            for (unsigned int c = 0; c < dim; ++c) pde->set_initial_condition(f, c, p, v[0], v[c]);
            for (unsigned int c = 0; c < dim; ++c) vals[f][(size_t)(c * lattice.N + node)] = v[c];
          }
        }
      }
    }
    for (unsigned int f : ic_fields) check(ppf_upload_state(handle, (int)f, 0, vals[f].data(), PPF_ORDER_LATTICE), "initial condition");
  }

  void update_dirichlet(unsigned int increment) {
    const double t = user_inputs->temporal_discretization.initial_time + increment * user_inputs->temporal_discretization.dt;
    SimulationTimer timer(user_inputs->temporal_discretization.dt, t);
    timer.set_increment(increment);
    for (size_t f = 0; f < field_attributes.size(); ++f) {
      if (!dirichlet_fields[f]) continue;
      if (adaptive) {
        // the engine evaluates set_dirichlet at the Dirichlet nodes of every mesh it builds,
        // at its current time
        check(ppf_set_dirichlet_function(handle, (int)f, &Problem::dirichlet_point, const_cast<Problem*>(this)),
              "Dirichlet function");
        continue;
      }
      const int ncomp = field_attributes[f].field_type == TensorRank::Vector ? (int)dim : 1;
      const long long len = ppf_field_length(handle, (int)f);
      std::vector<int> cmap((size_t)len);
      check(ppf_constraint_map(handle, (int)f, cmap.data()), "constraint map");
      std::vector<double> v((size_t)len, 0.0);
      const auto& bcs = user_inputs->boundary_parameters.boundary_condition_list.at(field_attributes[f].name);
      for (int c = 0; c < ncomp; ++c) {
        auto cc = bcs.component_constraints.find((unsigned)c);
        if (cc == bcs.component_constraints.end()) continue;
        for (long long node = 0; node < lattice.N; ++node) {
          const long long gi = c * lattice.N + node;
          if (cmap[(size_t)gi] >= 0) continue;
          // first Dirichlet boundary of this component that contains the node
          long long ijk[3] = {node % lattice.nn[0], (node / lattice.nn[0]) % lattice.nn[1],
                              node / ((long long)lattice.nn[0] * lattice.nn[1])};
          unsigned int bid = 0;
          for (unsigned int b = 0; b < 2 * dim; ++b) {
            auto it = cc->second.find(b);
            if (it == cc->second.end() || it->second != Condition::Dirichlet) continue;
            const long long at = (b % 2 == 0) ? 0 : lattice.nn[b / 2] - 1;
            if (ijk[b / 2] == at) {
              bid = b;
              break;
            }
          }
          number s[3] = {0, 0, 0};
          const dealii::Point<dim> p = node_point(node);
          if (ncomp == 1) {
            pde->set_dirichlet((unsigned)f, bid, 0, p, timer, s[0], s[0]);
            v[(size_t)gi] = s[0];
          } else {
            pde->set_dirichlet((unsigned)f, bid, (unsigned)c, p, timer, s[0], s[c]);
            v[(size_t)gi] = s[c];
          }
        }
      }
      check(ppf_set_dirichlet_values(handle, (int)f, v.data()), "Dirichlet values");
    }
  }

  void write_output(unsigned int increment) {
    const auto& O = user_inputs->output_parameters;
    const unsigned int n = user_inputs->temporal_discretization.n_increments;
    const int digits = n == 0 ? 1 : (int)std::floor(std::log10((double)n)) + 1;
    std::ostringstream inc;
    inc << std::setw(digits) << std::setfill('0') << increment;
    std::vector<std::vector<double>> sol(field_attributes.size());
    std::vector<output::OutputField> of;
    // the handle's own order: the lattice on uniform meshes, the DoF list on adaptive ones
    const long long N = ppf_n_nodes(handle);
    std::vector<double> invm((size_t)N);
    check(ppf_invm(handle, invm.data()), "inverse mass");
    double t = 0.0;
    unsigned int cur = 0;
    ppf_get_time(handle, &cur, &t);
    t = user_inputs->temporal_discretization.initial_time + increment * user_inputs->temporal_discretization.dt;
    std::cout << "Iteration " << increment << " Time " << t << std::endl;
    for (size_t f = 0; f < field_attributes.size(); ++f) {
      sol[f].resize((size_t)ppf_field_length(handle, (int)f));
      check(ppf_download_solution(handle, (int)f, sol[f].data(), PPF_ORDER_NATIVE), "download");
      const int ncomp = field_attributes[f].field_type == TensorRank::Vector ? (int)dim : 1;
      double l2 = 0.0;
      for (double x : sol[f]) l2 += x * x;
      std::cout << "  Field index " << f << " name " << field_attributes[f].name << " l2-norm " << std::sqrt(l2)
                << " integrated value ";
      for (int c = 0; c < ncomp; ++c) {
        double integral = 0.0;
        for (long long i = 0; i < N; ++i)
          if (invm[(size_t)i] > 0.0) integral += sol[f][(size_t)(c * N + i)] / invm[(size_t)i];
        std::cout << integral << (c + 1 < ncomp ? " " : "");
      }
      std::cout << std::endl;
      if (!O.output_fields.empty() && !O.output_fields.count(field_attributes[f].name)) continue;
      of.push_back({field_attributes[f].name, ncomp, sol[f].data()});
    }
    std::cout << std::endl;
    const std::string prefix = (std::filesystem::path(O.folder) / O.file_name).string();
    output::CellList cl;
    std::vector<int> cells, cell_dofs;
    if (adaptive) {
      cl.ncells = ppf_n_cells(handle);
      cells.resize((size_t)(4 * cl.ncells));
      cell_dofs.resize((size_t)(cl.ncells * (long long)std::pow(degree + 1, dim)));
      check(ppf_cells(handle, cells.data()), "cells");
      check(ppf_cell_dofs(handle, cell_dofs.data()), "cell DoFs");
      cl.cells = cells.data();
      cl.cell_dofs = cell_dofs.data();
      cl.N = N;
      const auto& rm = user_inputs->spatial_discretization.rectangular_mesh;
      for (unsigned int d = 0; d < dim; ++d) {
        cl.subdivisions[d] = (int)rm.subdivisions[d];
        cl.size[d] = rm.size[d] - rm.lower_bound[d];
      }
    }
    output::VTUWriter writer = adaptive ? output::VTUWriter(lattice, cl, O.patch_subdivisions)
                                        : output::VTUWriter(lattice, O.patch_subdivisions);
    if (O.file_type == FieldOutputParameters::PVTU) {
      const std::string piece = prefix + "_" + inc.str() + ".0.vtu";
      writer.write(piece, of, t, increment);
      output::write_pvtu_record(prefix + "_" + inc.str() + ".pvtu", piece, of);
    } else {
      if (O.file_type != FieldOutputParameters::VTU && !warned_format) {
        std::cout << "note: writing VTU output in place of the requested file type" << std::endl;
        warned_format = true;
      }
      writer.write(prefix + "_" + inc.str() + ".vtu", of, t, increment);
    }
  }

  std::vector<FieldAttributes> field_attributes;
  std::vector<SolveBlock> solve_blocks;
  const UserInputParameters<dim>* user_inputs;
  PhaseFieldTools<dim>* pf_tools;
  const Base* pde;
  Base* hooks = nullptr;  // the same operator, for its non-const hooks and user stop
  bool has_hooks = false;
  const unsigned char* object_source = nullptr;
  size_t object_size = 0;
  bool has_lhs = false;
  ppf_cell_launch_fn launcher = nullptr;
  ppf_handle handle = nullptr;
  output::Lattice lattice;
  std::vector<bool> dirichlet_fields;
  bool time_dependent = false;
  bool adaptive = false;
  bool warned_format = false;
};

PRISMS_PF_END_NAMESPACE

#pragma pop_macro("compute_lhs")
#pragma pop_macro("compute_rhs")

#pragma pop_macro("post_solve_block")
#pragma pop_macro("pre_solve_block")
