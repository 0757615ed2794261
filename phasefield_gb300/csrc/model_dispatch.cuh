// Instantiation and dispatch of cell_kernel<PDE, dim, degree, mode, number> for one operator
// set. Each built-in model's translation unit includes this with its own template.
#pragma once

#include <cstring>
#include <string>

#include <prismspf/gpu/launch.cuh>

#include "runtime.h"

namespace ppf {

template <template <unsigned int, unsigned int, typename> class M, int dim, int degree, int mode, typename number>
cudaError_t launch_one(const CellLaunch& P, const void* obj, size_t smem, cudaStream_t s) {
  return launch_cell_kernel<M<dim, degree, number>, dim, degree, mode, number>(P, obj, smem, s);
}

// precision: 0 = FP64, 1 = FP32 (LHS modes only, for mixed-precision smoothing); a mode with
// MODE_AMR set launches the adaptive-mesh kernel and `P` is the base of an AmrCellLaunch
template <template <unsigned int, unsigned int, typename> class M, bool with_lhs>
cudaError_t dispatch_launch(int dim, int degree, int mode, int precision, const CellLaunch& P, const void* obj,
                            size_t smem, cudaStream_t s) {
#define PPF_CASE(D, K)                                                                   \
  if (dim == D && degree == K) {                                                         \
    if (precision == 0 && mode == (MODE_RHS | MODE_AMR))                                 \
      return launch_amr_operator<M<D, K, double>, D, K, MODE_RHS>(&P, obj, smem, s);     \
    if constexpr (with_lhs) {                                                            \
      if (precision == 0 && mode == (MODE_LHS | MODE_AMR))                               \
        return launch_amr_operator<M<D, K, double>, D, K, MODE_LHS>(&P, obj, smem, s);   \
      if (precision == 0 && mode == MODE_LHS) return launch_one<M, D, K, MODE_LHS, double>(P, obj, smem, s);   \
      if (precision == 0 && mode == MODE_DIAG) return launch_one<M, D, K, MODE_DIAG, double>(P, obj, smem, s); \
      if (precision == 1 && mode == MODE_LHS) return launch_one<M, D, K, MODE_LHS, float>(P, obj, smem, s);    \
      if (precision == 1 && mode == MODE_DIAG) return launch_one<M, D, K, MODE_DIAG, float>(P, obj, smem, s);  \
    }                                                                                    \
    if (precision == 0 && mode == MODE_RHS) return launch_one<M, D, K, MODE_RHS, double>(P, obj, smem, s);     \
    return cudaErrorInvalidValue;                                                        \
  }
  PPF_CASE(2, 1)
  PPF_CASE(2, 2)
  PPF_CASE(2, 3)
  PPF_CASE(2, 4)
  PPF_CASE(3, 1)
  PPF_CASE(3, 2)
  PPF_CASE(3, 3)
  PPF_CASE(3, 4)
#undef PPF_CASE
  return cudaErrorInvalidValue;
}

}  // namespace ppf
