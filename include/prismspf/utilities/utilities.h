// Process set-up helper (reference: include/prismspf/utilities/utilities.h:39-60). The
// engine runs one process per GPU without MPI, so construction and destruction do nothing
// beyond keeping the reference's call sites valid.
#pragma once

#include <prismspf/config.h>

PRISMS_PF_BEGIN_NAMESPACE

class MPIInitFinalize {
 public:
  MPIInitFinalize(int& /*argc*/, char**& /*argv*/, unsigned int /*max_n_threads*/ = 0) {}
  MPIInitFinalize(const MPIInitFinalize&) = delete;
  MPIInitFinalize& operator=(const MPIInitFinalize&) = delete;
};

PRISMS_PF_END_NAMESPACE
