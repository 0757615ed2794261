// Warp-resident cell kernel for FP64 Q1/Q2 operators on the uniform lattice: the measured
// alternative to cell_kernel's thread-block tiles, run for an operator's left-hand side when the
// operator asks for it (`cell_warp_lhs`, the elasticity operator does) and for every FP64 Q1/Q2
// launch with PPF_CELL_KERNEL=warp.
//
// The same per-cell work as cell_kernel (gather -> user callback per quadrature point ->
// integrate -> condensed scatter; MFOperator::compute_local_operator,
// src/solvers/mf_operator.cc:34-80, with FieldContainer::reinit_and_eval /
// integrate_and_distribute, include/prismspf/core/field_container.h:794-882), laid out so that
// every cell lives inside one warp:
//   * a warp owns 32 / (k+1)^dim whole cells (Q2 3-D: one cell on lanes 0-26; Q2 2-D: three
//     cells on lanes 0-26; Q1: four or eight cells on all 32 lanes), one lane per (cell,
//     quadrature point), and walks cell groups in a grid-stride loop of its own;
//   * everything a cell shares (its nodal values, their fixed-point copies and block exponents,
//     the submitted terms) sits in the warp's own shared-memory region, so the only
//     synchronisation is __syncwarp: no block barrier after the tables are staged;
//   * the per-cell block exponents of the exact integer contractions are warp reductions (one
//     redux.sync for a 27-lane cell, a shuffle butterfly for 4- and 8-lane cells, a shared
//     atomicMax for 9-lane cells);
//   * lattice indices are 32-bit (fewer than 2^31 entries per vector, as the int32 constraint
//     maps already require).
// The FieldContainer the callback sees is unchanged: its context points at the warp's region
// (row stride 32 lanes). Measured on the Cahn-Hilliard Q2 3-D benchmark it ties cell_kernel
// (the idle lanes 27-31 of a Q2 3-D warp cost as much FP64 and issue bandwidth as the barriers
// they remove), so cell_kernel stays the default there; the elasticity left-hand side, whose
// 64-register callback leaves the thread-block tiles at 24 warps per SM, gains 8 % here.
#pragma once

#include <cuda_runtime.h>

#include <prismspf/gpu/cell_kernel.cuh>

#pragma push_macro("compute_rhs")
#pragma push_macro("compute_lhs")
#undef compute_rhs
#undef compute_lhs

namespace ppf {

// An operator may ask for a register budget of this kernel through `static constexpr int
// cell_warp_min_blocks` (resident 256-thread blocks per SM); the default is 6 (40 registers).
template <class PDE, class = void>
struct CellWarpMinBlocks {
  static constexpr int value = 6;
};
template <class PDE>
struct CellWarpMinBlocks<PDE, std::void_t<decltype(PDE::cell_warp_min_blocks)>> {
  static constexpr int value = PDE::cell_warp_min_blocks;
};

// Largest block exponent among the lanes of a cell. `slot` points at the cell exponents of
// this row (one int per cell of the warp); the shared-memory path expects them zeroed.
template <int nq, int cpw>
__device__ __forceinline__ int cell_exponent_max(int e, int* slot, int lc) {
  if constexpr (cpw == 1) {
    return __reduce_max_sync(0xffffffffu, e);
  } else if constexpr ((nq & (nq - 1)) == 0) {
    // cells start at multiples of nq (a power of two): the butterfly stays inside the cell
#pragma unroll
    for (int off = nq / 2; off > 0; off >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
    return e;
  } else {
    if (lc < cpw) atomicMax(slot + lc, e);
    __syncwarp();
    return lc < cpw ? slot[lc] : 0;
  }
}

template <int dim, int degree>
__device__ __forceinline__ double integrate_row_warp(const pg::CellTables<dim, degree, double>* tab,
                                                     const double* outs, int rv, bool has_v, bool has_g, int lane,
                                                     int cbase, int q, int qa, int qb, int qc) {
  constexpr int n = degree + 1;
  double r = has_v ? outs[rv * 32 + lane] : 0.0;
  if (has_g) {
#pragma unroll
    for (int d = 0; d < dim; ++d) {
      const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
      const int id = d == 0 ? qa : (d == 1 ? qb : qc);
      const double* g = outs + (rv + 1 + d) * 32 + cbase + (q - id * sd);
      const double* w = tab->jdt[d][q];
#pragma unroll
      for (int j = 0; j < n; ++j) r = fma(w[j], g[j * sd], r);
    }
  }
  return r;
}

// the submitted gradient terms of row rv already converted in place to fixed point with the
// cell's block exponent E of that output component
template <int dim, int degree>
__device__ __forceinline__ double integrate_row_warp_fx(const pg::CellTables<dim, degree, double>* tab,
                                                        const double* outs, int rv, bool has_v, bool has_g,
                                                        int lane, int cbase, int q, int qa, int qb, int qc, int E) {
  constexpr int n = degree + 1;
  namespace fx = pg::fx;
  double r = has_v ? outs[rv * 32 + lane] : 0.0;
  if (has_g) {
    if (E == fx::EXP_NONFINITE) return fx::quiet_nan();
    const long long* gx = reinterpret_cast<const long long*>(outs);
    const int lsb = E - 1023 - fx::TOP_TERMS;
    long long sum = 0;
    double rg = 0.0;
    const bool cubic = tab->fx_cubic != 0;
#pragma unroll
    for (int d = 0; d < dim; ++d) {
      const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
      const int id = d == 0 ? qa : (d == 1 ? qb : qc);
      const long long* g = gx + (rv + 1 + d) * 32 + cbase + (q - id * sd);
      long long p = fx::line_integral<n>(id, g[0], g[sd], n > 2 ? g[2 * sd] : 0ll);
      p = (long long)((unsigned long long)p << tab->wo_sh[d][q]);
      if (cubic) sum += p;
      else rg += fx::to_double(p, lsb + tab->ik[d], tab->isig[d]);
    }
    if (cubic) rg = fx::to_double(sum, lsb + tab->ik[0], tab->isig[0]);
    r += rg;
  }
  return r;
}

// FXINT: compile the fixed-point integration path (contraction modes 2 and 3)
template <class PDE, int dim, int degree, int MODE, bool FXINT>
__global__ void __launch_bounds__(WarpShape<dim, degree>::threads, CellWarpMinBlocks<PDE>::value)
    cell_kernel_warp(const __grid_constant__ CellLaunch P, const __grid_constant__ PDE pde) {
  static_assert(degree <= 2 && MODE != MODE_DIAG, "the warp kernel covers FP64 Q1/Q2 RHS and LHS launches");
  using W = WarpShape<dim, degree>;
  using Tab = pg::CellTables<dim, degree, double>;
  constexpr int n = W::n, nq = W::nq, cpw = W::cpw, k = degree;
  constexpr bool SMEM_MAX = !(cpw == 1 || (nq & (nq - 1)) == 0);
  namespace fx = pg::fx;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Tab* tab = reinterpret_cast<Tab*>(smem_raw);
  {
    const int nwords = (int)(sizeof(Tab) / 4);
    const unsigned int* src = reinterpret_cast<const unsigned int*>(P.tables);
    unsigned int* dst = reinterpret_cast<unsigned int*>(tab);
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
  }
  const Tab* gtab = reinterpret_cast<const Tab*>(P.tables);
  const bool fx_tab = gtab->fx != 0;
  const unsigned int fx_rows = gtab->fx_rows;
  const bool fx_on = fx_tab && P.fx_deriv != 0;
  const bool fx_int = FXINT && fx_tab && P.fx_int != 0;
  const SimulationTimer timer = P.timer_dev ? *P.timer_dev : P.timer;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wbase = smem_raw + (sizeof(Tab) + 15) / 16 * 16 +
                         (size_t)warp * warp_region_bytes<dim, degree>(P.nrows_in, P.nrows_out);
  double* vals = reinterpret_cast<double*>(wbase);
  long long* vfx = reinterpret_cast<long long*>(vals + P.nrows_in * 32);
  double* outs = reinterpret_cast<double*>(vfx + P.nrows_in * 32);
  int* ex_in = reinterpret_cast<int*>(outs + P.nrows_out * 32);
  int* ex_out = ex_in + P.nrows_in * cpw;

  const int lc = lane / nq;
  const int q = lane - lc * nq;
  const int cbase = lc * nq;
  const int qa = q % n;
  const int qb = dim > 1 ? (q / n) % n : 0;
  const int qc = dim > 2 ? q / (n * n) : 0;
  const bool lane_ok = lane < W::lanes;
  const bool writer = q == 0 && lc < cpw;  // writes the cell's exponents
  pg::fx::FastDiv div0, div1;
  div0.init((unsigned int)P.nc[0]);
  div1.init((unsigned int)P.nc[1]);
  const unsigned int nn0 = (unsigned int)P.nn[0], nn1 = (unsigned int)P.nn[1];
  const unsigned int N = (unsigned int)P.N;
  const unsigned int ncells = (unsigned int)P.ncells;
  const unsigned int ngroups = (ncells + cpw - 1) / cpw;
  __syncthreads();  // tables staged

  for (unsigned int g = blockIdx.x * W::warps + warp; g < ngroups; g += gridDim.x * W::warps) {
    const unsigned int cell = g * cpw + lc;
    const bool active = lane_ok && cell < ncells;
    int cx = 0, cy = 0, cz = 0;
    unsigned int node = 0;
    if (active) {
      const unsigned int q0 = div0.div(cell);
      cx = (int)(cell - q0 * div0.d);
      if (dim == 2) cy = (int)q0;
      if (dim > 2) {
        const unsigned int q1 = div1.div(q0);
        cy = (int)(q0 - q1 * div1.d);
        cz = (int)q1;
      }
      node = ((unsigned int)(k * cz + qc) * nn1 + (unsigned int)(k * cy + qb)) * nn0 + (unsigned int)(k * cx + qa);
    }
    __syncwarp();  // the previous group is done with this warp's region
    if constexpr (SMEM_MAX) {
      if (writer) {
        for (int r = 0; r < P.nrows_in; ++r) ex_in[r * cpw + lc] = 0;
        for (int r = 0; r < P.nrows_out; ++r) ex_out[r * cpw + lc] = 0;
      }
      __syncwarp();
    }

    // gather (read_dof_values_plain, or read_dof_values for a constrained src), with the
    // fixed-point copy of every row read as a gradient
    {
      int row = 0;
#pragma unroll
      for (int s = 0; s < pg::MAX_SLOTS; ++s) {
        if (s < P.nslots) {
          const SlotDesc& sd = P.slots[s];
          const double* ptr = static_cast<const double*>(sd.ptr);
          for (int c = 0; c < sd.ncomp; ++c) {
            double v = 0.0;
            if (active) {
              const unsigned int idx = node + (unsigned int)c * N;
              if (sd.constrained_read) {
                const int m = __ldg(sd.cmap + idx);
                const double own = __ldg(ptr + idx);
                v = m == (int)idx ? own : (m >= 0 ? __ldg(ptr + m) : 0.0);
              } else {
                v = __ldg(ptr + idx);
              }
            }
            const int r = row + c;
            vals[r * 32 + lane] = v;
            if (fx_on && ((fx_rows >> r) & 1u)) {
              const int E = cell_exponent_max<nq, cpw>(active ? fx::exponent(v) : 0, ex_in + r * cpw, lc);
              if constexpr (!SMEM_MAX) {
                if (writer) ex_in[r * cpw + lc] = E;
              }
              vfx[r * 32 + lane] = E == fx::EXP_NONFINITE ? 0ll : fx::to_fixed(v, E, fx::TOP_VALUES);
            } else if (writer) {
              ex_in[r * cpw + lc] = -1;  // no fixed-point copy: FP64 contractions for this row
            }
          }
          row += sd.ncomp;
        }
      }
    }
    for (int r = 0; r < P.nrows_out; ++r) outs[r * 32 + lane] = 0.0;
    __syncwarp();  // the cell's nodal values, fixed-point copies and exponents are visible

    pg::CellCtx<dim, degree, double> ctx;
    ctx.tab = tab;
    ctx.vals = vals;
    ctx.outs = outs;
    ctx.stride = 32;
    ctx.lc = lc;
    ctx.q = q;
    ctx.cell[0] = cx;
    ctx.cell[1] = cy;
    ctx.cell[2] = cz;
    ctx.err = P.err;
    ctx.submitted = 0;
    if (fx_on) {
      ctx.vals_fx = vfx;
      ctx.ex_in = ex_in;
      ctx.cpb = cpw;
    }
    if (active) {
      FieldContainer<dim, degree, double> fc(ctx);
      if constexpr (MODE == MODE_LHS) pde.compute_lhs(fc, timer, P.block_id);
      else pde.compute_rhs(fc, timer, P.block_id);
    }
    const int flags = __reduce_or_sync(0xffffffffu, ctx.submitted);

    if constexpr (FXINT) {
      if (fx_int) {
        // submitted gradient terms -> fixed point in place, one block exponent per cell and
        // output component (rows of component c of output o: value, then dim gradient rows)
#pragma unroll
        for (int o = 0; o < pg::MAX_OUTS; ++o) {
          if (o < P.nout && (flags & (2 << (2 * o)))) {
            for (int c = 0; c < P.outs[o].ncomp; ++c) {
              const int rv = tab->out_row0[o] + c * (1 + dim);
              double gv[dim];
              int e = 0;
#pragma unroll
              for (int d = 0; d < dim; ++d) {
                gv[d] = outs[(rv + 1 + d) * 32 + lane];
                e = max(e, fx::exponent(gv[d]));
              }
              const int E = cell_exponent_max<nq, cpw>(e, ex_out + rv * cpw, lc);
              if constexpr (!SMEM_MAX) {
                if (writer) ex_out[rv * cpw + lc] = E;
              }
#pragma unroll
              for (int d = 0; d < dim; ++d)
                reinterpret_cast<long long*>(outs)[(rv + 1 + d) * 32 + lane] =
                    E == fx::EXP_NONFINITE ? 0ll : fx::to_fixed(gv[d], E, fx::TOP_TERMS);
            }
          }
        }
      }
    }
    __syncwarp();  // the submitted terms (and their exponents) are visible

    if (active) {
#pragma unroll
      for (int o = 0; o < pg::MAX_OUTS; ++o) {
        if (o < P.nout) {
          const OutDesc& od = P.outs[o];
          const bool has_v = flags & (1 << (2 * o));
          const bool has_g = flags & (2 << (2 * o));
          if (!(has_v || has_g)) continue;
          const int row0 = tab->out_row0[o];
          for (int c = 0; c < od.ncomp; ++c) {
            const int rv = row0 + c * (1 + dim);
            double r;
            if (FXINT && fx_int)
              r = integrate_row_warp_fx<dim, degree>(tab, outs, rv, has_v, has_g, lane, cbase, q, qa, qb, qc,
                                                     ex_out[rv * cpw + lc]);
            else
              r = integrate_row_warp<dim, degree>(tab, outs, rv, has_v, has_g, lane, cbase, q, qa, qb, qc);
            const unsigned int idx = node + (unsigned int)c * N;
            const int target = od.cmap ? __ldg(od.cmap + idx) : (int)idx;
            if (target >= 0) atomicAdd(static_cast<double*>(od.acc) + target, r);
          }
        }
      }
    }
  }
}

template <class PDE, int dim, int degree, int mode, bool FXINT>
cudaError_t launch_cell_kernel_warp_impl(const CellLaunch& P, const void* obj, size_t smem, cudaStream_t s) {
  using W = WarpShape<dim, degree>;
  auto kern = cell_kernel_warp<PDE, dim, degree, mode, FXINT>;
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
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, W::threads, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
  }
  const long long groups = (P.ncells + W::cpw - 1) / W::cpw;
  const long long blocks_needed = (groups + W::warps - 1) / W::warps;
  long long grid = (long long)sms * occ;
  if (grid > blocks_needed) grid = blocks_needed;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, W::threads, smem, s>>>(P, *reinterpret_cast<const PDE*>(obj));
  return cudaGetLastError();
}

}  // namespace ppf

#pragma pop_macro("compute_lhs")
#pragma pop_macro("compute_rhs")
