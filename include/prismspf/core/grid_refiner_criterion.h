// Refinement criteria of adaptive meshes (include/prismspf/core/grid_refiner_criterion.h of the
// reference, same names and semantics): a field is a reason to refine a cell when its value lies
// in the open range (value_lower_bound, value_upper_bound) or its gradient magnitude exceeds
// gradient_lower_bound at one of the cell's quadrature points.
#pragma once

#include <cfloat>
#include <string>

#include <prismspf/config.h>

PRISMS_PF_BEGIN_NAMESPACE

enum RefinementFlags : unsigned int {
  Nothing = 0,
  Value = 0x0001,
  Gradient = 0x0002,
};

inline constexpr RefinementFlags operator|(RefinementFlags a, RefinementFlags b) {
  return static_cast<RefinementFlags>(static_cast<unsigned int>(a) | static_cast<unsigned int>(b));
}
inline constexpr RefinementFlags& operator|=(RefinementFlags& a, RefinementFlags b) { return a = a | b; }
inline constexpr RefinementFlags operator&(RefinementFlags a, RefinementFlags b) {
  return static_cast<RefinementFlags>(static_cast<unsigned int>(a) & static_cast<unsigned int>(b));
}
inline constexpr RefinementFlags& operator&=(RefinementFlags& a, RefinementFlags b) { return a = a & b; }

struct RefinementCriterion {
  explicit RefinementCriterion(const RefinementFlags& c = RefinementFlags::Nothing, const double& vlo = DBL_MAX,
                               const double& vhi = DBL_MAX, const double& glo = DBL_MAX)
      : criterion(c), value_lower_bound(vlo), value_upper_bound(vhi), gradient_lower_bound(glo) {}

  [[nodiscard]] bool value_in_open_range(double v) const { return v > value_lower_bound && v < value_upper_bound; }
  [[nodiscard]] bool gradient_magnitude_above_threshold(double g) const { return g > gradient_lower_bound; }

  [[nodiscard]] std::string criterion_string() const {
    const bool v = (criterion & RefinementFlags::Value) != 0U, g = (criterion & RefinementFlags::Gradient) != 0U;
    if (criterion == RefinementFlags::Nothing) return "None";
    if (v && g) return "Value and gradient";
    if (v) return "Value";
    if (g) return "Gradient";
    return "Unknown criterion";
  }

  RefinementFlags criterion = RefinementFlags::Nothing;
  double value_lower_bound = DBL_MAX;
  double value_upper_bound = DBL_MAX;
  double gradient_lower_bound = DBL_MAX;
};

PRISMS_PF_END_NAMESPACE
