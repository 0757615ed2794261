// Test driver: parses a parameter file with the drop-in UserInputParameters<dim> and prints
// what it read as JSON (one object), or {"error": "..."} when the file is rejected.
// Also prints make_dependency_set results for dependency strings given after the file name
// ("--deps name1,name2 str1 str2 ...").
#include <prismspf/core/dependencies.h>
#include <prismspf/user_inputs/user_input_parameters.h>

#include <iomanip>
#include <iostream>
#include <sstream>

using namespace prismspf;

static std::string esc(const std::string& s) {
  std::string o;
  for (char c : s) o += (c == '"' || c == '\\') ? std::string("\\") + c : std::string(1, c);
  return o;
}

template <unsigned int dim>
static int dump(const char* file) {
  UserInputParameters<dim> u(file);
  std::ostringstream o;
  o << std::setprecision(17) << "{";
  const auto& m = u.spatial_discretization.rectangular_mesh;
  o << "\"size\": [";
  for (unsigned d = 0; d < dim; ++d) o << (d ? ", " : "") << m.size[d];
  o << "], \"lower\": [";
  for (unsigned d = 0; d < dim; ++d) o << (d ? ", " : "") << m.lower_bound[d];
  o << "], \"subdivisions\": [";
  for (unsigned d = 0; d < dim; ++d) o << (d ? ", " : "") << m.subdivisions[d];
  o << "], \"periodic\": [";
  bool first = true;
  for (unsigned p : m.periodic_directions) o << (first ? "" : ", ") << p, first = false;
  o << "], \"refinement\": " << u.spatial_discretization.global_refinement;
  o << ", \"adaptivity\": " << (u.spatial_discretization.has_adaptivity ? "true" : "false");
  o << ", \"dt\": " << u.temporal_discretization.dt << ", \"n_increments\": " << u.temporal_discretization.n_increments;
  o << ", \"outputs\": [";
  first = true;
  for (unsigned x : u.output_parameters.output_list) o << (first ? "" : ", ") << x, first = false;
  o << "], \"file_type\": " << (int)u.output_parameters.file_type << ", \"folder\": \"" << esc(u.output_parameters.folder)
    << "\", \"file_name\": \"" << esc(u.output_parameters.file_name) << "\"";
  o << ", \"seed\": " << u.misc_parameters.random_seed << ", \"rng_first\": " << u.misc_parameters.rng();
  o << ", \"bcs\": {";
  first = true;
  for (const auto& [name, set] : u.boundary_parameters.boundary_condition_list) {
    o << (first ? "" : ", ") << "\"" << esc(name) << "\": {";
    first = false;
    bool f2 = true;
    for (const auto& [comp, conds] : set.component_constraints) {
      o << (f2 ? "" : ", ") << "\"" << comp << "\": [";
      f2 = false;
      bool f3 = true;
      for (const auto& [b, c] : conds) o << (f3 ? "" : ", ") << (int)c, f3 = false;
      o << "]";
    }
    o << "}";
  }
  o << "}, \"linear\": {";
  first = true;
  for (const auto& [id, L] : u.linear_solve_parameters.linear_solvers) {
    o << (first ? "" : ", ") << "\"" << id << "\": {\"tolerance_type\": " << (int)L.tolerance_type
      << ", \"tolerance\": " << L.tolerance << ", \"max_iterations\": " << L.max_iterations
      << ", \"preconditioner\": " << (int)L.preconditioner << ", \"mg_depth\": " << L.mg_depth
      << ", \"smoother_degree\": " << L.chebyshev_parameters.degree
      << ", \"smoothing_range\": " << L.chebyshev_parameters.smoothing_range
      << ", \"eig_cg_iterations\": " << L.chebyshev_parameters.eig_cg_n_iterations << "}";
    first = false;
  }
  o << "}, \"constants\": {";
  first = true;
  for (const auto& [name, v] : u.user_constants.model_constants) {
    o << (first ? "" : ", ") << "\"" << esc(name) << "\": ";
    first = false;
    if (auto* d = std::get_if<double>(&v)) o << *d;
    else if (auto* i = std::get_if<int>(&v)) o << "{\"int\": " << *i << "}";
    else if (auto* b = std::get_if<bool>(&v)) o << (*b ? "true" : "false");
    else if (auto* s = std::get_if<std::string>(&v)) o << "\"" << esc(*s) << "\"";
    else if (auto* t = std::get_if<dealii::Tensor<1, dim, double>>(&v)) {
      o << "[";
      for (unsigned d = 0; d < dim; ++d) o << (d ? ", " : "") << (*t)[d];
      o << "]";
    } else if (auto* t2 = std::get_if<dealii::Tensor<2, dim, double>>(&v)) {
      o << "[";
      for (unsigned i = 0; i < dim; ++i) {
        o << (i ? ", [" : "[");
        for (unsigned j = 0; j < dim; ++j) o << (j ? ", " : "") << (*t2)[i][j];
        o << "]";
      }
      o << "]";
    } else {
      const auto C = u.user_constants.get_elasticity_tensor(name);
      const int nv = UserConstants<dim>::voigt;
      o << "{\"voigt\": [";
      for (int i = 0; i < nv; ++i) {
        o << (i ? ", [" : "[");
        for (int j = 0; j < nv; ++j) o << (j ? ", " : "") << C[i][j];
        o << "]";
      }
      o << "]}";
    }
  }
  o << "}, \"not_applied\": " << u.not_applied.size() << "}";
  std::cout << o.str() << std::endl;
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 3 && std::string(argv[1]) == "--deps") {
    std::vector<FieldAttributes> fields;
    std::stringstream names(argv[2]);
    std::string n;
    while (std::getline(names, n, ',')) fields.emplace_back(n);
    std::set<std::string> strs;
    for (int i = 3; i < argc; ++i) strs.insert(argv[i]);
    try {
      const DependencyMap m = make_dependency_set(fields, strs);
      std::cout << "{";
      bool first = true;
      for (const auto& [f, d] : m) {
        std::cout << (first ? "" : ", ") << "\"" << f << "\": [" << (int)d.flag << ", " << (int)d.src_flag << ", [";
        for (size_t a = 0; a < d.old_flags.size(); ++a) std::cout << (a ? ", " : "") << (int)d.old_flags[a];
        std::cout << "]]";
        first = false;
      }
      std::cout << "}" << std::endl;
    } catch (std::exception& e) {
      std::cout << "{\"error\": \"" << esc(e.what()) << "\"}" << std::endl;
    }
    return 0;
  }
  if (argc != 3) {
    std::cerr << "usage: prm_dump <dim> <file.prm> | --deps <names> <strings...>" << std::endl;
    return 2;
  }
  try {
    const int dim = std::stoi(argv[1]);
    if (dim == 2) return dump<2>(argv[2]);
    if (dim == 3) return dump<3>(argv[2]);
    return dump<1>(argv[2]);
  } catch (std::exception& e) {
    std::cout << "{\"error\": \"" << esc(e.what()) << "\"}" << std::endl;
    return 0;
  }
}
