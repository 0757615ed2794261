// ORACLE — test infrastructure only (see oracle.cc). Not part of the product.
#pragma once

enum {
  ORC_MODEL_ALLEN_CAHN = 1,
  ORC_MODEL_CAHN_HILLIARD = 2,
  ORC_MODEL_ESHELBY = 3,
  ORC_MODEL_COUPLED_ACCH = 4,
  ORC_MODEL_ALLEN_CAHN_IMPLICIT = 5,
  ORC_MODEL_CAHN_HILLIARD_IMPLICIT = 6,
};

enum {
  ORC_TIMING_PRIMARY = 0,
  ORC_TIMING_SECONDARY = 1,
  ORC_TIMING_POSTPROCESS = 2,
};

enum {
  ORC_ERR_NAN = 2,
};
