// Instantiation and dispatch of cell_kernel<PDE, dim, degree, mode, number> for one operator
// set. Each built-in model's translation unit includes this with its own template.
#pragma once

#include <cstring>
#include <string>

#include "runtime.h"

namespace ppf {

template <template <unsigned int, unsigned int, typename> class M, int dim, int degree, int mode, typename number>
cudaError_t launch_one(const CellLaunch& P, const void* obj, size_t smem, cudaStream_t s) {
  using PDE = M<dim, degree, number>;
  using S = CellShape<dim, degree>;
  auto kern = cell_kernel<PDE, dim, degree, mode, number>;
  static size_t attr_smem = 0;
  static int occ = 0;
  static int sms = 0;
  if (smem > attr_smem) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_smem = smem;
    occ = 0;
  }
  if (occ == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, S::threads, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
  }
  const long long ntiles = (P.ncells + S::cpb - 1) / S::cpb;
  long long grid = (long long)sms * occ;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, S::threads, smem, s>>>(P, *reinterpret_cast<const PDE*>(obj));
  return cudaGetLastError();
}

// precision: 0 = FP64, 1 = FP32 (LHS modes only, for mixed-precision smoothing)
template <template <unsigned int, unsigned int, typename> class M, bool with_lhs>
cudaError_t dispatch_launch(int dim, int degree, int mode, int precision, const CellLaunch& P, const void* obj,
                            size_t smem, cudaStream_t s) {
#define PPF_CASE(D, K)                                                                   \
  if (dim == D && degree == K) {                                                         \
    if constexpr (with_lhs) {                                                            \
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
