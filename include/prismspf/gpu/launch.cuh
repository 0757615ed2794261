// Host-side launcher of cell_kernel<PDE, dim, degree, mode, number>: opts in to the dynamic
// shared memory the launch needs, sizes a persistent grid of (SM count x resident blocks per
// SM) blocks capped at the number of cell tiles, and launches on the given stream.
//
// Used by the library's built-in operators and by prismspf/core/problem.h for a user's
// CustomPDE, so both sides launch the kernel the same way. `obj` points to the host bytes of
// the operator object; they are passed to the kernel by value.
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include <prismspf/gpu/amr_cell_kernel.cuh>
#include <prismspf/gpu/cell_kernel.cuh>
#include <prismspf/gpu/cell_kernel_lanes.cuh>
#include <prismspf/gpu/cell_kernel_warp.cuh>

namespace ppf {

template <class PDE, int dim, int degree, int mode, typename number, bool FXINT>
cudaError_t launch_cell_kernel_impl(const CellLaunch& P, const void* obj, size_t smem, cudaStream_t s) {
  using S = CellShape<dim, degree>;
  auto kern = cell_kernel<PDE, dim, degree, mode, number, FXINT>;
  // the shared-memory opt-in and the occupancy hold per device: cached per device ordinal
  constexpr int MAX_DEVICES = 64;
  static size_t attr_smem_of[MAX_DEVICES] = {};
  static int occ_of[MAX_DEVICES] = {};
  static int sms_of[MAX_DEVICES] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  size_t& attr_smem = attr_smem_of[dev];
  int& occ = occ_of[dev];
  int& sms = sms_of[dev];
  if (smem > attr_smem) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_smem = smem;
    occ = 0;
  }
  if (occ == 0) {
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, S::threads, smem);
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

// An operator may run its FP64 Q1/Q2 left-hand side on the warp-resident kernel
// (cell_kernel_warp.cuh) through `static constexpr bool cell_warp_lhs = true`; everything else
// runs cell_kernel's thread-block tiles.
template <class PDE, class = void>
struct CellWarpLhs {
  static constexpr bool value = false;
};
template <class PDE>
struct CellWarpLhs<PDE, std::void_t<decltype(PDE::cell_warp_lhs)>> {
  static constexpr bool value = PDE::cell_warp_lhs;
};

// PPF_CELL_KERNEL=warp runs every FP64 Q1/Q2 RHS and LHS launch on the warp-resident kernel,
// PPF_CELL_KERNEL=block none; otherwise the operator's choice (0 operator, 1 warp, 2 block)
inline int cell_kernel_override() {
  static const int v = [] {
    const char* e = std::getenv("PPF_CELL_KERNEL");
    if (e && std::strcmp(e, "warp") == 0) return 1;
    if (e && std::strcmp(e, "block") == 0) return 2;
    return 0;
  }();
  return v;
}

template <class PDE, int mode>
inline bool use_warp_cell_kernel() {
  const int o = cell_kernel_override();
  if (o) return o == 1;
  return mode == MODE_LHS && CellWarpLhs<PDE>::value;
}

// launches the instantiation with the fixed-point integration path only when the launch asks
// for it (contraction modes 2 and 3 of FP64 Q1/Q2 operators)
template <class PDE, int dim, int degree, int mode, typename number>
cudaError_t launch_cell_kernel(const CellLaunch& P, const void* obj, size_t smem, cudaStream_t s) {
  if constexpr (std::is_same<number, float>::value && degree <= 2 && mode == MODE_LHS) {
    // FP32 left-hand sides (mixed-precision smoothing levels) on the lane layout when asked
    if (P.fx_lanes) {
      const cudaError_t e = launch_cell_kernel_lanes_f32_impl<PDE, dim, degree>(P, obj, s);
      if (e != cudaErrorNotSupported) return e;
    }
  }
  if constexpr (cell_fx_capable<dim, degree, number>() && mode != MODE_DIAG) {
    if (P.fx_lanes) {
      // the lane kernel when its rows and tile fit (and the host tables came with the launch),
      // else integer derivatives on the thread-block tiles
      const cudaError_t e = launch_cell_kernel_lanes_impl<PDE, dim, degree, mode>(P, obj, s);
      if (e != cudaErrorNotSupported) return e;
      return launch_cell_kernel_impl<PDE, dim, degree, mode, number, false>(P, obj, smem, s);
    }
    if (use_warp_cell_kernel<PDE, mode>() && smem >= cell_warp_smem_bytes<dim, degree>(P.nrows_in, P.nrows_out)) {
      if (P.fx_int) return launch_cell_kernel_warp_impl<PDE, dim, degree, mode, true>(P, obj, smem, s);
      return launch_cell_kernel_warp_impl<PDE, dim, degree, mode, false>(P, obj, smem, s);
    }
    if (P.fx_int) return launch_cell_kernel_impl<PDE, dim, degree, mode, number, true>(P, obj, smem, s);
  }
  return launch_cell_kernel_impl<PDE, dim, degree, mode, number, false>(P, obj, smem, s);
}

// The adaptive-mesh kernel for a mode without the MODE_AMR flag; `rec` is an AmrCellLaunch.
// Adaptive meshes exist for degrees 1 and 2 (nested Gauss-Lobatto points), so only those are
// instantiated.
template <class PDE, int dim, int degree, int mode>
cudaError_t launch_amr_operator(const void* rec, const void* obj, size_t smem, cudaStream_t s) {
  if constexpr (degree <= 2 && dim >= 2)
    return launch_amr_cell_kernel<PDE, dim, degree, mode, double>(*static_cast<const AmrCellLaunch*>(rec), obj, smem,
                                                                  s);
  else
    return cudaErrorInvalidValue;
}

}  // namespace ppf
