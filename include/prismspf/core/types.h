// Index and flag types shared by the host-side API (reference: include/prismspf/core/types.h).
#pragma once

#include <prismspf/config.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/dealii_shim.h>

PRISMS_PF_BEGIN_NAMESPACE

namespace Types {
using Index = unsigned int;
}  // namespace Types

namespace Numbers {
static const Types::Index invalid_index = static_cast<Types::Index>(-1);
static constexpr unsigned int default_subsections = 5;
}  // namespace Numbers

using EvalFlags = dealii::EvaluationFlags::EvaluationFlags;

PRISMS_PF_END_NAMESPACE
