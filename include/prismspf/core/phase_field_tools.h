// Tools handed to the user's operator (reference: include/prismspf/core/phase_field_tools.h).
#pragma once

#include <vector>

#include <prismspf/config.h>
#include <prismspf/nucleation/nucleus.h>

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim>
struct PhaseFieldTools {
  std::vector<Nucleus<dim>> nuclei_list;
};

PRISMS_PF_END_NAMESPACE
