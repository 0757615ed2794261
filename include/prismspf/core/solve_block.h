// Declarative solve block (reference: include/prismspf/core/solve_block.h:28-127): the
// fields a solver updates, how (SolveType), when (SolveTiming) and from which dependencies.
#pragma once

#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <prismspf/config.h>
#include <prismspf/core/dependencies.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/core/types.h>
#include <prismspf/user_inputs/solve_parameters.h>

PRISMS_PF_BEGIN_NAMESPACE

class SolveBlock {
 public:
  using EvalFlags = prismspf::EvalFlags;
  using FieldType = TensorRank;

  explicit SolveBlock(int _id = -1, SolveType _solve_type = Explicit, SolveTiming _solve_timing = Primary,
                      std::set<Types::Index> _field_indices = {}, DependencyMap _dependencies_rhs = {},
                      DependencyMap _dependencies_lhs = {})
      : id(_id),
        solve_type(_solve_type),
        solve_timing(_solve_timing),
        field_indices(std::move(_field_indices)),
        dependencies_rhs(std::move(_dependencies_rhs)),
        dependencies_lhs(std::move(_dependencies_lhs)) {}

  int id;
  SolveType solve_type;
  SolveTiming solve_timing;
  std::set<Types::Index> field_indices;
  DependencyMap dependencies_rhs;
  DependencyMap dependencies_lhs;
  LinearSolverParameters linear_solver_parameters;
  NonlinearSolverParameters nonlinear_solver_parameters;

  bool operator<(const SolveBlock& other) const { return id < other.id; }

  // the checks of SolveBlock::validate (solve_block.h:129-212) that apply to this engine
  void validate() const {
    if (solve_type != Constant && solve_type != Explicit && solve_type != Linear && solve_type != Newton)
      throw std::invalid_argument("A valid solve type must be selected (Constant | Explicit | Linear | Newton)");
    if (field_indices.empty()) throw std::invalid_argument("Solve blocks must manage at least 1 field");
    if (solve_type == Newton)
      for (unsigned int f : field_indices) {
        auto r = dependencies_rhs.find(f);
        auto l = dependencies_lhs.find(f);
        if (r == dependencies_rhs.end() || r->second.flag == EvalFlags::nothing)
          throw std::invalid_argument("Every field in a newton solve should appear in the residual (RHS) expression");
        if (l == dependencies_lhs.end() || l->second.src_flag == EvalFlags::nothing)
          throw std::invalid_argument(
              "Every field in a newton solve should appear as a Delta term in the residual Jacobian (LHS) expression");
      }
  }
};

PRISMS_PF_END_NAMESPACE
