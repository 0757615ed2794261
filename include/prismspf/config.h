// Namespace macros used by every PRISMS-PF header and application
// (reference: include/prismspf/config.h.in).
#pragma once

#define PRISMS_PF_BEGIN_NAMESPACE namespace prismspf {
#define PRISMS_PF_END_NAMESPACE }
