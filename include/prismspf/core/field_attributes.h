// Field declaration (reference: include/prismspf/core/field_attributes.h): a name, a tensor
// rank and the boundary conditions the parameter file attaches to it.
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <prismspf/config.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/core/types.h>
#include <prismspf/user_inputs/constraint_parameters.h>

PRISMS_PF_BEGIN_NAMESPACE

struct FieldAttributes {
  explicit FieldAttributes(std::string _name = "", TensorRank _field_type = TensorRank::Scalar,
                           BoundaryConditionSet _boundary_conditions = BoundaryConditionSet(),
                           bool _is_nucleation_rate_variable = false,
                           std::vector<Types::Index> _nucleating_field_indices = std::vector<Types::Index>())
      : name(std::move(_name)),
        field_type(_field_type),
        boundary_conditions(std::move(_boundary_conditions)),
        is_nucleation_rate_variable(_is_nucleation_rate_variable),
        nucleating_field_indices(std::move(_nucleating_field_indices)) {}

  std::string name;
  TensorRank field_type = TensorRank::Scalar;
  BoundaryConditionSet boundary_conditions;
  bool is_nucleation_rate_variable = false;
  std::vector<Types::Index> nucleating_field_indices;
};

inline std::map<std::string, Types::Index> field_index_map(const std::vector<FieldAttributes>& fields) {
  std::map<std::string, Types::Index> map;
  for (unsigned int i = 0; i < fields.size(); ++i) {
    if (map.count(fields[i].name)) throw std::invalid_argument("The names of the fields must be unique: " + fields[i].name);
    map[fields[i].name] = i;
  }
  return map;
}

PRISMS_PF_END_NAMESPACE
