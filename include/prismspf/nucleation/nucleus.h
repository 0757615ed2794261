// A seeded nucleus record (reference: include/prismspf/nucleation/nucleus.h). Stochastic
// nucleation is outside this engine; the type exists so PhaseFieldTools keeps its shape.
#pragma once

#include <prismspf/config.h>
#include <prismspf/dealii_shim.h>

PRISMS_PF_BEGIN_NAMESPACE

template <unsigned int dim>
struct Nucleus {
  unsigned int field_index = 0;
  dealii::Point<dim, double> location;
  double seed_time = 0.0;
  unsigned int seed_increment = 0;
};

PRISMS_PF_END_NAMESPACE
