// Parameters read from the .prm file (reference: include/prismspf/user_inputs/
// user_input_parameters.h:27-146 and the declare/assign pairs in src/user_inputs/*.cc):
// rectangular mesh and global refinement, time stepping, boundary conditions, linear solver
// parameters per solve block, output schedule, the random seed and the Model constants.
// Entry names and aliases are the reference's. Nucleation, checkpoint and initial-condition-file
// entries are read and reported as not applied (analytic initial conditions).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <map>
#include <random>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include <prismspf/config.h>
#include <prismspf/core/grid_refiner_criterion.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/dealii_shim.h>
#include <prismspf/user_inputs/constraint_parameters.h>
#include <prismspf/user_inputs/parameter_file.h>
#include <prismspf/user_inputs/solve_parameters.h>
#include <prismspf/user_inputs/user_constants.h>

PRISMS_PF_BEGIN_NAMESPACE

using RNGEngine = std::mt19937;

template <unsigned int dim>
struct RectangularMesh {
  // boundary ids in natural language
  enum Boundary { Left = 0, Right = 1, Top = 2, Bottom = 3, Front = 4, Back = 5 };

  dealii::Tensor<1, dim, double> size;         // upper bound per axis
  dealii::Tensor<1, dim, double> lower_bound;  // lower bound per axis
  std::vector<unsigned int> subdivisions = std::vector<unsigned int>(dim, 1);
  std::set<unsigned int> periodic_directions;
};

template <unsigned int dim>
struct SpatialDiscretization {
  RectangularMesh<dim> rectangular_mesh;
  unsigned int global_refinement = 0;
  bool has_adaptivity = false;
  unsigned int max_refinement = 0;
  unsigned int min_refinement = 0;
  unsigned int remeshing_period = UINT32_MAX;
  // refinement criteria by field name (spatial_discretization.cc:462-496)
  std::map<std::string, RefinementCriterion> refinement_criteria;

  // whether the increment is a remeshing increment (spatial_discretization.cc:608-611)
  [[nodiscard]] bool should_refine_mesh(unsigned int increment) const { return increment % remeshing_period == 0; }

  // Euclidean distance between two points (SpatialDiscretization::distance)
  template <typename T>
  T distance(const dealii::Point<dim, T>& a, const dealii::Point<dim, T>& b) const {
    return a.distance(b);
  }
};

struct TemporalDiscretization {
  double dt = 1.0;
  double initial_time = 0.0;
  unsigned int n_increments = 0;
};

struct FieldOutputParameters {
  enum OutputType { VTU, VTK, PVTU, XDMF };
  std::string folder = "solutions";
  std::string file_name = "solution";
  unsigned int patch_subdivisions = 0;
  OutputType file_type = VTU;
  std::set<unsigned int> output_list;
  std::set<std::string> output_fields;

  bool should_output(unsigned int increment) const { return output_list.count(increment) != 0; }
};

struct MiscellaneousParameters {
  unsigned int random_seed = 2025;
  mutable RNGEngine rng{random_seed};
  void set_random_seed(unsigned int seed) {
    random_seed = seed;
    rng.seed(random_seed);  // + MPI rank in the reference; one process here
  }
};

// output schedules (io_parameters.h:33-100)
inline void add_equal_spacing_outputs(unsigned int n_outputs, unsigned int n_increments, std::set<unsigned int>& out) {
  out.clear();
  if (n_increments == 0) {
    out.insert(0);
    return;
  }
  if (!n_outputs) return;
  const unsigned int period = std::max(1u, n_increments / n_outputs);
  for (unsigned int o = 0; o <= n_increments; o += period) out.insert(o);
}

inline void add_log_spacing_outputs(unsigned int n_outputs, unsigned int n_increments, std::set<unsigned int>& out) {
  out.clear();
  if (n_increments == 0) {
    out.insert(0);
    return;
  }
  if (!n_outputs) return;
  for (unsigned int o = 1; o <= n_outputs; ++o)
    out.insert((unsigned int)std::round(std::pow(double(n_increments), double(o) / double(n_outputs))));
}

inline void add_n_per_decade_outputs(unsigned int n_outputs, unsigned int n_increments, std::set<unsigned int>& out) {
  out.clear();
  if (n_increments == 0) {
    out.insert(0);
    return;
  }
  if (!n_outputs) return;
  out.insert(0);
  out.insert(1);
  for (unsigned int it = 2; it <= n_increments; ++it) {
    const auto decade = (unsigned int)std::ceil(std::log10(it));
    const auto step = (unsigned int)(std::pow(10, decade) / n_outputs);
    if (step != 0 && it % step == 0) out.insert(it);
  }
}

template <unsigned int dim>
class UserInputParameters {
 public:
  explicit UserInputParameters(const std::string& input_file_name) : parameters(input_file_name) { assign(); }

  // from text (tests and embedded configurations)
  static UserInputParameters from_string(const std::string& text) { return UserInputParameters(text, 0); }

  SpatialDiscretization<dim> spatial_discretization;
  TemporalDiscretization temporal_discretization;
  LinearSolveParameters linear_solve_parameters;
  NonlinearSolveParameters nonlinear_solve_parameters;
  FieldOutputParameters output_parameters;
  BoundaryParameters boundary_parameters;
  UserConstants<dim> user_constants;
  MiscellaneousParameters misc_parameters;
  // the nucleation-attempt schedule (nucleation_parameters.cc:25-29, 110-113): NucleationRate
  // blocks run on output increments and on increments divisible by the period
  struct NucleationSchedule {
    unsigned int nucleation_period = 2147483647u;
    bool should_attempt_nucleation(unsigned int increment) const { return increment % nucleation_period == 0; }
  } nucleation_parameters;
  std::vector<std::string> not_applied;  // entries read but without effect in this engine
  prm::ParameterFile parameters;

 private:
  UserInputParameters(const std::string& text, int) {
    parameters.parse(text);
    assign();
  }

  static std::vector<std::string> aliases(const std::string& n, std::vector<std::string> more = {}) {
    more.insert(more.begin(), n);
    return more;
  }

  void assign() {
    const prm::ParameterFile& P = parameters;
    // mesh (spatial_discretization.cc:210-300)
    const std::string mesh_type = P.get("", {"mesh type", "mesh_type"}, "rectangular");
    if (mesh_type != "rectangular") throw std::invalid_argument("only the rectangular mesh type is supported");
    const char axes[3] = {'x', 'y', 'z'};
    for (unsigned int i = 0; i < dim; ++i) {
      const std::string a(1, axes[i]);
      auto& m = spatial_discretization.rectangular_mesh;
      m.size[i] = prm::to_double(P.get("Rectangular mesh", {a + " size", "size " + a, a + " upper bound",
                                                            "upper bound " + a}, "0.0"));
      m.lower_bound[i] = prm::to_double(P.get("Rectangular mesh", {a + " lower bound", "lower bound " + a}, "0.0"));
      m.subdivisions[i] = (unsigned int)prm::to_int(P.get("Rectangular mesh", {a + " subdivisions",
                                                                               "subdivisions " + a}, "1"));
      if (prm::to_bool(P.get("Rectangular mesh", {a + " periodic", "periodic " + a}, "false")))
        m.periodic_directions.insert(i);
    }
    for (unsigned int i = dim; i < 3; ++i) {  // entries of the unused axes are allowed
      const std::string a(1, axes[i]);
      std::string dummy;
      P.find("Rectangular mesh", {a + " size", "size " + a, a + " upper bound", "upper bound " + a}, dummy);
      P.find("Rectangular mesh", {a + " lower bound", "lower bound " + a}, dummy);
      P.find("Rectangular mesh", {a + " subdivisions", "subdivisions " + a}, dummy);
      P.find("Rectangular mesh", {a + " periodic", "periodic " + a}, dummy);
    }
    spatial_discretization.global_refinement = (unsigned int)prm::to_int(P.get("", {"global refinement"}, "0"));
    spatial_discretization.has_adaptivity = prm::to_bool(P.get("", {"mesh adaptivity"}, "false"));
    spatial_discretization.max_refinement = (unsigned int)prm::to_int(P.get("", {"max refinement"}, "0"));
    spatial_discretization.min_refinement = (unsigned int)prm::to_int(P.get("", {"min refinement"}, "0"));
    {
      std::string v;
      if (P.find("", {"remeshing period"}, v)) spatial_discretization.remeshing_period = (unsigned int)prm::to_int(v);
    }
    // refinement criteria (spatial_discretization.cc:395-496): type none | value | gradient |
    // value_and_gradient for the listed fields
    for (const auto& sec : P.subsections_with_prefix("refinement criterion: ")) {
      P.mark_used_prefix(sec + "/");
      const std::string type = P.get(sec, {"type"}, "none");
      RefinementFlags flags = RefinementFlags::Nothing;
      if (type == "value") flags = RefinementFlags::Value;
      else if (type == "gradient") flags = RefinementFlags::Gradient;
      else if (type == "value_and_gradient") flags = RefinementFlags::Value | RefinementFlags::Gradient;
      else if (type != "none" && !type.empty()) throw std::invalid_argument(sec + ": unknown refinement criterion type " + type);
      const RefinementCriterion c(flags, prm::to_double(P.get(sec, {"value lower bound"}, "0.0")),
                                  prm::to_double(P.get(sec, {"value upper bound"}, "0.0")),
                                  prm::to_double(P.get(sec, {"gradient magnitude lower bound", "gradient lower bound"},
                                                       "2147483647")));
      for (const auto& name : prm::split_list(P.get(sec, {"variables"}, "")))
        if (!name.empty()) spatial_discretization.refinement_criteria[name] = c;
    }

    // time (temporal_discretization.cc:33-110)
    auto& T = temporal_discretization;
    T.n_increments = (unsigned int)prm::to_int(P.get(
        "", {"final increment", "number steps", "number of steps", "num steps", "n steps", "last increment",
             "end increment", "final_increment", "number_steps", "number_of_steps", "num_steps", "n_steps",
             "last_increment", "end_increment", "steps", "iterations", "final iteration", "max iteration",
             "increments"},
        "0"));
    T.dt = prm::to_double(P.get("", {"time step", "timestep", "time_step", "dt"}, "0.0"));
    T.initial_time = prm::to_double(P.get("", {"start time", "start_time", "t_0", "t0", "begin time", "begin_time"},
                                          "0.0"));
    const double final_time =
        prm::to_double(P.get("", {"end time", "end_time", "t_f", "tf", "final time", "final_time"}, "0.0"));
    if (final_time > 0.0) {
      if (T.initial_time > final_time) throw std::invalid_argument("Initial time must be less than or equal to final time.");
      T.n_increments = (unsigned int)std::ceil((final_time - T.initial_time) / T.dt);
    }
    if (T.n_increments != 0 && !(T.dt > 0.0))
      throw std::invalid_argument("Time step must be greater than 0 for transient problems.");

    // boundary conditions (constraint_parameters.cc:41-107)
    for (const auto& sec : P.subsections_with_prefix("boundary conditions: ")) {
      const auto names = prm::split_list(P.get(sec, {"variables"}, ""));
      const auto conds = prm::split_list(P.get(sec, {"conditions"}, ""));
      const bool td = prm::to_bool(P.get(sec, {"time dependent", "time_dependent"}, "false"));
      ComponentConditions cc;
      for (unsigned int b = 0; b < conds.size(); ++b) cc[b] = condition_from_string(conds[b]);
      for (const auto& fc : names) {
        std::string field = fc;
        std::set<unsigned int> comps;
        if (fc.size() > 2 && fc[fc.size() - 2] == ':' && (fc.back() == 'x' || fc.back() == 'y' || fc.back() == 'z')) {
          comps = {(unsigned int)(fc.back() - 'x')};
          field = fc.substr(0, fc.size() - 2);
        } else {
          for (unsigned int c = 0; c < dim; ++c) comps.insert(c);
        }
        for (unsigned int c : comps)
          if (c < dim) boundary_parameters.boundary_condition_list[field].component_constraints[c] = cc;
        boundary_parameters.boundary_condition_list[field].time_dependent = td;
      }
    }

    // linear solver parameters per block (solve_parameters.cc:280-330)
    for (const auto& sec : P.subsections_with_prefix("linear solver parameters: ")) {
      LinearSolverParameters L;
      L.solver_type = P.get(sec, {"solver type", "solver_type", "linear solver type", "linear_solver_type",
                                  "linear solver", "linear_solver", "type"}, "cg");
      const std::string tt = P.get(sec, {"tolerance type"}, "AbsoluteResidual");
      const char* tnames[] = {"AbsoluteResidual", "RMSEPerField", "IntegratedPerField", "RMSETotal",
                              "IntegratedTotal"};
      bool ok = false;
      for (int i = 0; i < 5; ++i)
        if (tt == tnames[i]) L.tolerance_type = SolverToleranceType(i), ok = true;
      if (!ok) throw std::invalid_argument("invalid tolerance type " + tt);
      L.tolerance = prm::to_double(P.get(sec, {"tolerance value", "tolerance"}, "1.0e-10"));
      L.max_iterations = (unsigned int)prm::to_int(P.get(sec, {"max iterations"}, "100"));
      L.mg_depth = (unsigned int)prm::to_int(P.get(sec, {"mg depth", "mg_depth"}, "1"));
      const std::string pc = P.get(sec, {"preconditioner type", "preconditioner_type", "preconditioner"}, "None");
      if (pc == "None" || pc == "none") L.preconditioner = PreconditionerType::None;
      else if (pc == "Chebyshev" || pc == "chebyshev") L.preconditioner = PreconditionerType::Chebyshev;
      else if (pc == "GMG" || pc == "gmg" || pc == "MG" || pc == "mg" || pc == "multigrid")
        L.preconditioner = PreconditionerType::GMG;
      else throw std::invalid_argument("invalid preconditioner type " + pc);
      L.chebyshev_parameters.smoothing_range = prm::to_double(P.get(sec + "/Chebyshev", {"smoothing range"}, "15.0"));
      L.chebyshev_parameters.degree = (unsigned int)prm::to_int(P.get(sec + "/Chebyshev", {"smoother degree"}, "5"));
      L.chebyshev_parameters.eig_cg_n_iterations =
          (unsigned int)prm::to_int(P.get(sec + "/Chebyshev", {"eigenvalue cg iterations"}, "10"));
      for (const char* other : {"/Richardson/", "/BiCGStab/", "/GMRES/"}) P.mark_used_prefix(sec + other);
      for (const auto& id : prm::split_list(P.get(sec, {"solver_ids", "solve blocks", "solve_blocks",
                                                          "solve block ids", "solve_block_ids", "solver ids"}, "")))
        linear_solve_parameters.linear_solvers[(unsigned int)prm::to_int(id)] = L;
    }
    // Newton parameters (solve_parameters.cc:350-470)
    for (const auto& sec : P.subsections_with_prefix("newton solver parameters: ")) {
      NonlinearSolverParameters N;
      N.max_iterations = (unsigned int)prm::to_int(P.get(sec, {"max iterations"}, "100"));
      N.tolerance_value = prm::to_double(P.get(sec, {"tolerance value", "tolerance"}, "1.0e-10"));
      N.step_length = prm::to_double(P.get(sec, {"step size"}, "1.0"));
      for (const auto& id : prm::split_list(P.get(sec, {"solver_ids", "solve blocks", "solve_blocks",
                                                          "solve block ids", "solve_block_ids", "solver ids"}, "")))
        nonlinear_solve_parameters.nonlinear_solvers[(unsigned int)prm::to_int(id)] = N;
      P.mark_used_prefix(sec + "/");
    }

    // output (io_parameters.cc:10-140)
    auto& O = output_parameters;
    O.folder = P.get("output", {"directory", "folder name"}, "solutions");
    O.file_name = P.get("output", {"file name"}, "solution");
    O.patch_subdivisions = (unsigned int)prm::to_int(P.get("output", {"subdivisions"}, "0"));
    const std::string ft = P.get("output", {"file type"}, "vtu");
    if (ft == "vtu") O.file_type = FieldOutputParameters::VTU;
    else if (ft == "pvtu") O.file_type = FieldOutputParameters::PVTU;
    else if (ft == "vtk") O.file_type = FieldOutputParameters::VTK;
    else if (ft == "xdmf") O.file_type = FieldOutputParameters::XDMF;
    else throw std::invalid_argument("invalid output file type " + ft);
    P.get("output", {"compression level"}, "default");
    for (const auto& v : prm::split_list(P.get("output", {"variables"}, ""))) O.output_fields.insert(v);
    const std::string condition = P.get("output", {"condition"}, "EQUAL_SPACING");
    const unsigned int n_out = (unsigned int)prm::to_int(P.get("output", {"number"}, "10"));
    if (condition == "EQUAL_SPACING") add_equal_spacing_outputs(n_out, T.n_increments, O.output_list);
    else if (condition == "LOG_SPACING") add_log_spacing_outputs(n_out, T.n_increments, O.output_list);
    else if (condition == "N_PER_DECADE") add_n_per_decade_outputs(n_out, T.n_increments, O.output_list);
    else throw std::invalid_argument("invalid output condition " + condition);
    for (const auto& v : prm::split_list(P.get("output", {"list"}, "0"))) O.output_list.insert((unsigned)prm::to_int(v));

    // miscellaneous (miscellaneous_parameters.cc:10-48)
    misc_parameters.set_random_seed((unsigned int)prm::to_int(P.get("miscellaneous", {"random seed"}, "2025")));

    // the nucleation-attempt period decides when NucleationRate blocks run; the other
    // nucleation entries drive stochastic nucleation, which this engine does not do
    {
      const long long period = prm::to_int(P.get("nucleation", {"nucleation period", "nucleation_period"},
                                                 "2147483647"));
      if (period < 1) throw std::invalid_argument("nucleation period must be at least 1");
      nucleation_parameters.nucleation_period = (unsigned int)period;
      bool other = false;
      for (const auto& [k, v] : P.entries)
        other |= k.rfind("nucleation/", 0) == 0 && k != "nucleation/nucleation period" &&
                 k != "nucleation/nucleation_period";
      if (other) {
        P.mark_used_prefix("nucleation/");
        not_applied.push_back("nucleation");
      }
    }
    // entries of subsystems outside this engine
    for (const char* sec : {"checkpoint/"}) {
      bool any = false;
      for (const auto& [k, v] : P.entries) any |= k.rfind(sec, 0) == 0;
      if (any) {
        P.mark_used_prefix(sec);
        not_applied.push_back(std::string(sec, std::string(sec).size() - 1));
      }
    }
    for (const auto& sec : P.subsections_with_prefix("initial condition file: ")) {
      P.mark_used_prefix(sec + "/");
      not_applied.push_back(sec);
    }
    {
      std::string v;
      if (P.find("", {"read initial conditions from file"}, v) && prm::to_bool(v))
        not_applied.push_back("read initial conditions from file");
    }
    for (const auto& sec : P.subsections_with_prefix("nucleation criterion: ")) {
      P.mark_used_prefix(sec + "/");
      not_applied.push_back(sec);
    }

    // Model constants (user_constants.h:967-1000)
    for (const auto& name : P.constant_order) user_constants.add_user_constant(name, P.model_constants.at(name));

    const auto unknown = P.unused();
    if (!unknown.empty()) {
      std::string msg = "unknown parameter file entries:";
      for (const auto& u : unknown) msg += " '" + u + "'";
      throw std::invalid_argument(msg);
    }
  }
};

PRISMS_PF_END_NAMESPACE
