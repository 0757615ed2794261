// Dependency sets of a solve block (reference: include/prismspf/core/dependencies.h:134-213).
//
// make_dependency_set parses strings such as "n", "grad(old_1(n))", "hess(c)", "lap(c)",
// "hessdiag(c)", "div(u)", "symgrad(u)", "curl(u)" and "src(u)" / "change(u)" /
// "trial(u)" / "lhs(u)" into per-field evaluation flags for the current value, the SRC
// (linear-solve trial) vector and the old ages old_1 .. old_6. Unrecognised strings throw.
#pragma once

#include <algorithm>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <prismspf/config.h>
#include <prismspf/core/field_attributes.h>
#include <prismspf/core/types.h>

PRISMS_PF_BEGIN_NAMESPACE

struct Dependency {
  EvalFlags flag = EvalFlags::nothing;
  EvalFlags src_flag = EvalFlags::nothing;
  std::vector<EvalFlags> old_flags;

  explicit Dependency(EvalFlags _flag = EvalFlags::nothing, EvalFlags _src_flag = EvalFlags::nothing,
                      const std::vector<EvalFlags>& _old_flags = {})
      : flag(_flag), src_flag(_src_flag), old_flags(_old_flags) {}

  Dependency& operator|=(const Dependency& other) {
    flag |= other.flag;
    src_flag |= other.src_flag;
    if (other.old_flags.size() > old_flags.size()) old_flags.resize(other.old_flags.size(), EvalFlags::nothing);
    for (size_t i = 0; i < other.old_flags.size(); ++i) old_flags[i] |= other.old_flags[i];
    return *this;
  }
  Dependency operator|(const Dependency& other) const {
    Dependency r = *this;
    r |= other;
    return r;
  }
  Dependency& operator&=(const Dependency& other) {
    flag &= other.flag;
    src_flag &= other.src_flag;
    old_flags.resize(std::min(old_flags.size(), other.old_flags.size()));
    for (size_t i = 0; i < old_flags.size(); ++i) old_flags[i] &= other.old_flags[i];
    return *this;
  }
  Dependency operator&(const Dependency& other) const {
    Dependency r = *this;
    r &= other;
    return r;
  }
};

using DependencyMap = std::map<Types::Index, Dependency>;

constexpr unsigned int default_max_checked_age = 6;

inline DependencyMap make_dependency_set(const std::vector<FieldAttributes>& field_attributes,
                                         std::set<std::string> dependency_strings,
                                         unsigned int max_checked_age = default_max_checked_age) {
  // operator wrappers and the flag each one asks for
  static const std::pair<std::pair<const char*, const char*>, EvalFlags> wrappers[] = {
      {{"", ""}, EvalFlags::values},               {{"grad(", ")"}, EvalFlags::gradients},
      {{"hess(", ")"}, EvalFlags::hessians},       {{"hessdiag(", ")"}, EvalFlags::hessians},
      {{"lap(", ")"}, EvalFlags::hessians},        {{"div(", ")"}, EvalFlags::gradients},
      {{"symgrad(", ")"}, EvalFlags::gradients},   {{"curl(", ")"}, EvalFlags::gradients},
  };
  static const char* const src_names[] = {"src(", "change(", "trial(", "lhs("};
  DependencyMap result;
  auto take = [&](const std::string& s) {
    auto it = dependency_strings.find(s);
    if (it == dependency_strings.end()) return false;
    dependency_strings.erase(it);
    return true;
  };
  for (unsigned int i = 0; i < field_attributes.size(); ++i) {
    const std::string& name = field_attributes[i].name;
    for (const auto& [wrap, flag] : wrappers) {
      const std::string pre = wrap.first, post = wrap.second;
      if (take(pre + name + post)) result[i].flag |= flag;
      for (const char* src : src_names)
        if (take(pre + src + name + ")" + post)) result[i].src_flag |= flag;
      for (unsigned int age = 0; age < max_checked_age; ++age)
        if (take(pre + "old_" + std::to_string(age + 1) + "(" + name + ")" + post)) {
          auto& d = result[i];
          if (d.old_flags.size() < age + 1) d.old_flags.resize(age + 1, EvalFlags::nothing);
          d.old_flags[age] |= flag;
        }
    }
  }
  if (!dependency_strings.empty()) {
    std::string msg = "The following dependencies were not recognized:";
    for (const auto& s : dependency_strings) msg += " " + s;
    throw std::invalid_argument(msg);
  }
  return result;
}

PRISMS_PF_END_NAMESPACE
