// Boundary-condition parameters (reference: include/prismspf/user_inputs/constraint_parameters.h,
// src/user_inputs/constraint_parameters.cc:41-107): one Condition per boundary id
// (x- = 0, x+ = 1, y- = 2, y+ = 3, z- = 4, z+ = 5) for each component of each field.
#pragma once

#include <map>
#include <stdexcept>
#include <string>

#include <prismspf/config.h>
#include <prismspf/core/type_enums.h>

PRISMS_PF_BEGIN_NAMESPACE

enum Condition { Natural, Dirichlet, Neumann, Periodic };

inline Condition condition_from_string(const std::string& s) {
  if (s == "Natural") return Condition::Natural;
  if (s == "Dirichlet") return Condition::Dirichlet;
  if (s == "Neumann") return Condition::Neumann;
  if (s == "Periodic") return Condition::Periodic;
  throw std::invalid_argument("Invalid boundary condition " + s);
}

// boundary id -> condition
using ComponentConditions = std::map<unsigned int, Condition>;

struct BoundaryConditionSet {
  // component -> conditions
  std::map<unsigned int, ComponentConditions> component_constraints;
  bool time_dependent = false;
};

struct BoundaryParameters {
  // field name -> its boundary-condition set
  std::map<std::string, BoundaryConditionSet> boundary_condition_list;
};

PRISMS_PF_END_NAMESPACE
