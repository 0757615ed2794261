// Matrix-free cell kernel: gather -> evaluate -> user callback per quadrature point ->
// integrate -> condensed scatter, for one solve block on a uniform hyper-rectangle mesh.
//
// Restates the per-cell work of MFOperator::compute_local_operator
// (src/solvers/mf_operator.cc:34-80) with FieldContainer::reinit_and_eval /
// integrate_and_distribute (include/prismspf/core/field_container.h:794-882) as one GPU
// kernel, plus the diagonal probe of MFOperator::compute_local_field_diagonal
// (src/solvers/mf_operator.cc:147-218):
//   * DoF vectors are stored in lattice order (x fastest) with periodic images kept, so the
//     nodes of cell (cx,cy,cz) are a dense (k+1)^dim box of the lattice: the gather needs no
//     index map. Constraint maps are int32 arrays over the same index space:
//     cmap[i] = i (free), = master (periodic image), = -1-j (Dirichlet row j).
//   * one thread per (cell, quadrature point); cells_per_block cells per thread block; the
//     block walks cell tiles in a grid-stride loop so the per-launch tables are staged into
//     shared memory once per resident block;
//   * with Gauss-Lobatto collocation, values at quadrature points are the nodal values and
//     gradients are 1-D contractions (FieldContainer::deriv);
//   * integration is the transposed contraction over the pre-weighted submitted terms;
//   * distribute_local_to_global: rows constrained to a master add into the master,
//     Dirichlet rows are dropped; contributions of neighbouring cells meet through
//     atomicAdd into a zeroed accumulator (the finalize kernels apply invM and constraints).
//   * MODE_DIAG replaces the SRC dependency of each block field by unit probes on one cell
//     node at a time (identity in every component, as the reference submits
//     identity<Rank>()) and keeps the integrated entry at the probed node.
//   * FP64 Q1/Q2 launches contract exactly in 64-bit integers (prismspf/gpu/fixed_point.cuh):
//     rows read as gradients get a fixed-point copy with a per-cell block exponent, the
//     derivatives are integer line sums rounded once, and with fx_int the submitted gradient
//     terms are integrated the same way (else in FP64 with jdt); the launch record selects the
//     split, which the engine times per operator.
// `number` is the arithmetic type (double for the drop-in, float for mixed-precision
// multigrid smoothing).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include <prismspf/core/field_container.h>

// prismspf/core/pde_operator_base.h re-declares the callback names as macros for user
// classes; the kernel calls them by their plain names.
#pragma push_macro("compute_rhs")
#pragma push_macro("compute_lhs")
#undef compute_rhs
#undef compute_lhs

// minimum resident blocks per SM the cell kernels are compiled for (register budget)
#ifndef PPF_CELL_MIN_BLOCKS
#define PPF_CELL_MIN_BLOCKS 1
#endif

namespace ppf {

// An operator may ask for a register budget through `static constexpr int cell_min_blocks`
// (resident blocks per SM); otherwise the kernels are compiled for PPF_CELL_MIN_BLOCKS.
template <class PDE, class = void>
struct CellMinBlocks {
  static constexpr int value = PPF_CELL_MIN_BLOCKS;
};
template <class PDE>
struct CellMinBlocks<PDE, std::void_t<decltype(PDE::cell_min_blocks)>> {
  static constexpr int value = PDE::cell_min_blocks;
};

using prismspf::FieldContainer;
using prismspf::SimulationTimer;
namespace pg = prismspf::gpu;

enum CellMode { MODE_RHS = 0, MODE_LHS = 1, MODE_DIAG = 2 };

struct SlotDesc {
  const void* ptr;    // component-major vector (ncomp * N) of the kernel's number type
  const int* cmap;    // constraint map, used when constrained_read
  int ncomp;
  int constrained_read;  // homogeneous constrained read (FEEvaluation::read_dof_values)
  int is_src;            // the SRC dependency of a block field (probed in MODE_DIAG)
  int out_index;         // block output the SRC slot belongs to (MODE_DIAG)
};

struct OutDesc {
  void* acc;         // accumulator (ncomp * N), zeroed before the launch
  const int* cmap;   // destination constraint map (condensation)
  int ncomp;
};

struct CellLaunch {
  int nc[3];
  int nn[3];
  long long N;       // lattice nodes per component
  long long ncells;
  int nslots;
  SlotDesc slots[pg::MAX_SLOTS];
  int nout;
  OutDesc outs[pg::MAX_OUTS];
  int nrows_in;      // sum of slot components
  int nrows_out;     // sum over outputs of ncomp * (1 + dim)
  const void* tables;  // device copy of CellTables<dim,degree,number>
  SimulationTimer timer;
  const SimulationTimer* timer_dev;  // when set (graph replays), the timer is read from here
  unsigned int block_id;
  int* err;
  // with integer contractions on in the tables: fx_deriv takes the derivatives in fixed point
  // (else FP64 from the nodal values), fx_int integrates in fixed point (else FP64 with jdt)
  int fx_deriv;
  int fx_int;
  // the lane kernel (prismspf/gpu/cell_kernel_lanes.cuh): all-integer contractions of an FP64
  // Q1/Q2 operator on cubic cells, when the tables allow it (fx_lanes); it takes the host copy
  // of `tables` (tables_host) as a kernel parameter
  int fx_lanes;
  const void* tables_host;
};

template <int dim, int degree>
struct CellShape {
  static constexpr int n = degree + 1;
  static constexpr int nq = pg::ipow(n, dim);
  static constexpr int cpb = (256 / nq) > 0 ? (256 / nq) : 1;  // cells per thread block
  static constexpr int threads = cpb * nq;
};

// FP64 Q1/Q2 kernels contract in 64-bit fixed point (prismspf/gpu/fixed_point.cuh) when the
// launch's tables enable it; their shared memory then also holds the fixed-point nodal values
// and the per-cell block exponents of the value rows and of the output components.
template <int dim, int degree, typename number>
__host__ __device__ constexpr bool cell_fx_capable() {
  return std::is_same<number, double>::value && degree <= 2;
}

// Shape of the warp-resident alternative kernel (prismspf/gpu/cell_kernel_warp.cuh): whole
// cells per warp, 8 warps per thread block.
template <int dim, int degree>
struct WarpShape {
  static constexpr int n = degree + 1;
  static constexpr int nq = pg::ipow(n, dim);
  static constexpr int cpw = 32 / nq;       // cells per warp
  static constexpr int lanes = cpw * nq;    // lanes holding a (cell, quadrature point)
  static constexpr int warps = 8;           // warps per thread block
  static constexpr int threads = 32 * warps;
};

// bytes of one warp's region: nodal values, their fixed-point copies and the submitted terms
// (32 lanes each), then the block exponents of the value rows and output components per cell
template <int dim, int degree>
__host__ __device__ constexpr size_t warp_region_bytes(int nrows_in, int nrows_out) {
  using W = WarpShape<dim, degree>;
  return (8 * 32 * (size_t)(2 * nrows_in + nrows_out) + 4 * (size_t)W::cpw * (size_t)(nrows_in + nrows_out) + 15) /
         16 * 16;
}

template <int dim, int degree>
__host__ __device__ constexpr size_t cell_warp_smem_bytes(int nrows_in, int nrows_out) {
  using W = WarpShape<dim, degree>;
  return (sizeof(pg::CellTables<dim, degree, double>) + 15) / 16 * 16 +
         W::warps * warp_region_bytes<dim, degree>(nrows_in, nrows_out);
}

// Dynamic shared memory of a launch: enough for cell_kernel and, for FP64 Q1/Q2, for the
// warp-resident kernel as well (the launcher picks either).
template <int dim, int degree, typename number>
__host__ __device__ inline size_t cell_smem_bytes(int nrows_in, int nrows_out) {
  using S = CellShape<dim, degree>;
  size_t tab = (sizeof(pg::CellTables<dim, degree, number>) + 15) / 16 * 16;
  size_t b = tab + sizeof(number) * (size_t)(nrows_in + nrows_out) * S::threads + 16;
  if (cell_fx_capable<dim, degree, number>()) {
    b += sizeof(long long) * (size_t)nrows_in * S::threads + sizeof(int) * (size_t)(nrows_in + nrows_out) * S::cpb;
    const size_t w = cell_warp_smem_bytes<dim, degree>(nrows_in, nrows_out);
    if (w > b) b = w;
  }
  return b;
}

template <int dim, int degree, typename number>
__device__ __forceinline__ number integrate_row(const pg::CellTables<dim, degree, number>* tab, const number* outs,
                                                int rv, bool has_v, bool has_g, int t, int lc, int q, int qa, int qb,
                                                int qc) {
  using S = CellShape<dim, degree>;
  constexpr int n = S::n, nq = S::nq;
  number r = has_v ? outs[rv * S::threads + t] : number(0);
  if (has_g) {
#pragma unroll
    for (int d = 0; d < dim; ++d) {
      const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
      const int id = d == 0 ? qa : (d == 1 ? qb : qc);
      const number* g = outs + (rv + 1 + d) * S::threads + lc * nq + (q - id * sd);
      const number* w = tab->jdt[d][q];
#pragma unroll
      for (int j = 0; j < n; ++j) r = fma(w[j], g[j * sd], r);
    }
  }
  return r;
}

// integrate_row with the submitted gradient terms already converted in place to fixed point
// (block exponent E of the output component): per direction the exact integer line sum with
// the weights iint, times the other directions' weights (a shift), rounded once with the
// scale c_d = JxW / (h_d w_int...) of the integer weights.
template <int dim, int degree>
__device__ __forceinline__ double integrate_row_fx(const pg::CellTables<dim, degree, double>* tab, const double* outs,
                                                   int rv, bool has_v, bool has_g, int t, int lc, int q, int qa, int qb,
                                                   int qc, int E) {
  using S = CellShape<dim, degree>;
  constexpr int n = S::n, nq = S::nq;
  namespace fx = pg::fx;
  double r = has_v ? outs[rv * S::threads + t] : 0.0;
  if (has_g) {
    if (E == fx::EXP_NONFINITE) return fx::quiet_nan();
    const long long* gx = reinterpret_cast<const long long*>(outs);
    const int lsb = E - 1023 - fx::TOP_TERMS;
    long long sum = 0;
    double rg = 0.0;
#pragma unroll
    for (int d = 0; d < dim; ++d) {
      const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
      const int id = d == 0 ? qa : (d == 1 ? qb : qc);
      const long long* g = gx + (rv + 1 + d) * S::threads + lc * nq + (q - id * sd);
      long long p = fx::line_integral<n>(id, g[0], g[sd], n > 2 ? g[2 * sd] : 0ll);
      p = (long long)((unsigned long long)p << tab->wo_sh[d][q]);
      if (tab->fx_cubic) sum += p;
      else rg += fx::to_double(p, lsb + tab->ik[d], tab->isig[d]);
    }
    if (tab->fx_cubic) rg = fx::to_double(sum, lsb + tab->ik[0], tab->isig[0]);
    r += rg;
  }
  return r;
}

// FXINT: compile the fixed-point integration path (modes 2 and 3); the mode-1 instantiation
// leaves it out, which keeps its register budget for the derivative path
template <class PDE, int dim, int degree, int MODE, typename number, bool FXINT = false>
__global__ void __launch_bounds__(CellShape<dim, degree>::threads, CellMinBlocks<PDE>::value)
    cell_kernel(const __grid_constant__ CellLaunch P, const __grid_constant__ PDE pde) {
  using S = CellShape<dim, degree>;
  using Tab = pg::CellTables<dim, degree, number>;
  constexpr int n = S::n, nq = S::nq, cpb = S::cpb, k = degree;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Tab* tab = reinterpret_cast<Tab*>(smem_raw);
  number* vals = reinterpret_cast<number*>(smem_raw + (sizeof(Tab) + 15) / 16 * 16);
  number* outs = vals + P.nrows_in * S::threads;
  __shared__ int sflags;
  // integer contractions: enabled by the launch's tables, and only with the shared memory for them
  constexpr bool FXC = cell_fx_capable<dim, degree, number>() && MODE != MODE_DIAG;
  long long* vals_fx = reinterpret_cast<long long*>(outs + P.nrows_out * S::threads);
  int* ex_in = reinterpret_cast<int*>(vals_fx + P.nrows_in * S::threads);
  int* ex_out = ex_in + P.nrows_in * cpb;
  bool fx_on = false, fx_int = false;  // fx_on: fixed-point derivatives
  unsigned int tab_fx_rows = 0;
  if constexpr (FXC) {
    unsigned int dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const Tab* gtab = reinterpret_cast<const Tab*>(P.tables);
    const bool fx_ok =
        gtab->fx != 0 && dyn >= (unsigned int)cell_smem_bytes<dim, degree, number>(P.nrows_in, P.nrows_out);
    tab_fx_rows = gtab->fx_rows;
    fx_on = fx_ok && P.fx_deriv != 0;
    if constexpr (FXINT) fx_int = fx_ok && P.fx_int != 0;
  }
  // cell coordinates by multiply-high division (cell indices stay below 2^31: DoF indices are int)
  pg::fx::FastDiv div0, div1;
  div0.init((unsigned int)P.nc[0]);
  div1.init((unsigned int)P.nc[1]);

  // stage the tables once per resident block
  {
    const int nwords = (int)(sizeof(Tab) / 4);
    const unsigned int* src = reinterpret_cast<const unsigned int*>(P.tables);
    unsigned int* dst = reinterpret_cast<unsigned int*>(tab);
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
  }

  const int t = threadIdx.x;
  const int lc = t / nq;
  const int q = t - lc * nq;
  const int qa = q % n;
  const int qb = dim > 1 ? (q / n) % n : 0;
  const int qc = dim > 2 ? q / (n * n) : 0;
  const long long ntiles = (P.ncells + cpb - 1) / cpb;

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long cell = tile * cpb + lc;
    const bool active = cell < P.ncells;
    int cx = 0, cy = 0, cz = 0;
    long long node = 0;
    if (active) {
      const unsigned int cl = (unsigned int)cell;
      const unsigned int q0 = div0.div(cl);
      cx = (int)(cl - q0 * div0.d);
      if (dim == 2) cy = (int)q0;
      if (dim > 2) {
        const unsigned int q1 = div1.div(q0);
        cy = (int)(q0 - q1 * div1.d);
        cz = (int)q1;
      }
      node = ((long long)(k * cz + qc) * P.nn[1] + (k * cy + qb)) * P.nn[0] + (k * cx + qa);
    }
    if constexpr (FXC) {
      // the value-row exponents were last read by the previous tile's callbacks; rows without a
      // fixed-point copy keep -1
      if (fx_on)
        for (int i = t; i < P.nrows_in * cpb; i += S::threads) ex_in[i] = ((tab_fx_rows >> (i / cpb)) & 1u) ? 0 : -1;
    }
    __syncthreads();  // tables staged; previous tile finished with vals/outs/sflags

    // gather (read_dof_values_plain, or read_dof_values for constrained src); in MODE_DIAG
    // the SRC rows are written by the probe loop below
    {
      int row = 0;
#pragma unroll
      for (int s = 0; s < pg::MAX_SLOTS; ++s) {
        if (s < P.nslots) {
          const SlotDesc& sd = P.slots[s];
          if (!(MODE == MODE_DIAG && sd.is_src)) {
            const number* ptr = static_cast<const number*>(sd.ptr);
            for (int c = 0; c < sd.ncomp; ++c) {
              number v = number(0);
              if (active) {
                const long long idx = node + c * P.N;
                if (sd.constrained_read) {
                  // the value load issues with the map load: almost every entry is free, so
                  // the dependent second load is only paid on constrained entries
                  const int m = __ldg(sd.cmap + idx);
                  const number own = __ldg(ptr + idx);
                  v = m == (int)idx ? own : (m >= 0 ? __ldg(ptr + m) : number(0));
                } else {
                  v = __ldg(ptr + idx);
                }
              }
              vals[(row + c) * S::threads + t] = v;
              if constexpr (FXC) {
                if (fx_on && ((tab_fx_rows >> (row + c)) & 1u)) atomicMax(&ex_in[(row + c) * cpb + lc], pg::fx::exponent(v));
              }
            }
          }
          row += sd.ncomp;
        }
      }
    }

    if constexpr (MODE != MODE_DIAG) {
      if constexpr (FXC) {
        if (fx_on) {
          __syncthreads();  // block exponents of the value rows complete
          for (int r = 0; r < P.nrows_in; ++r) {
            const int E = ex_in[r * cpb + lc];
            if (E >= 0 && E != pg::fx::EXP_NONFINITE)
              vals_fx[r * S::threads + t] = pg::fx::to_fixed(vals[r * S::threads + t], E, pg::fx::TOP_VALUES);
          }
        }
        if (fx_int)
          for (int i = t; i < P.nrows_out * cpb; i += S::threads) ex_out[i] = 0;
      }
      if (t == 0) sflags = 0;
      for (int r = 0; r < P.nrows_out; ++r) outs[r * S::threads + t] = number(0);
      __syncthreads();

      pg::CellCtx<dim, degree, number> ctx;
      ctx.tab = tab;
      ctx.vals = vals;
      ctx.outs = outs;
      ctx.stride = S::threads;
      ctx.lc = lc;
      ctx.q = q;
      ctx.cell[0] = cx;
      ctx.cell[1] = cy;
      ctx.cell[2] = cz;
      ctx.err = P.err;
      ctx.submitted = 0;
      if constexpr (FXC) {
        if (fx_on) {
          ctx.vals_fx = vals_fx;
          ctx.ex_in = ex_in;
          ctx.cpb = cpb;
        }
      }
      if (active) {
        FieldContainer<dim, degree, number> fc(ctx);
        const SimulationTimer timer = P.timer_dev ? *P.timer_dev : P.timer;
        if constexpr (MODE == MODE_LHS) pde.compute_lhs(fc, timer, P.block_id);
        else pde.compute_rhs(fc, timer, P.block_id);
        if (ctx.submitted) atomicOr(&sflags, ctx.submitted);
      }
      __syncthreads();
      const int flags = sflags;

      if constexpr (FXC) {
        if (fx_int) {
          // submitted gradient terms -> fixed point in place, one block exponent per cell and
          // output component (rows of component c of output o: value, then dim gradient rows)
          for (int o = 0; o < P.nout; ++o)
            if (flags & (2 << (2 * o)))
              for (int c = 0; c < P.outs[o].ncomp; ++c) {
                const int rv = tab->out_row0[o] + c * (1 + dim);
                int e = 0;
#pragma unroll
                for (int d = 0; d < dim; ++d) e = max(e, pg::fx::exponent(outs[(rv + 1 + d) * S::threads + t]));
                atomicMax(&ex_out[rv * cpb + lc], e);
              }
          __syncthreads();
          for (int o = 0; o < P.nout; ++o)
            if (flags & (2 << (2 * o)))
              for (int c = 0; c < P.outs[o].ncomp; ++c) {
                const int rv = tab->out_row0[o] + c * (1 + dim);
                const int E = ex_out[rv * cpb + lc];
#pragma unroll
                for (int d = 0; d < dim; ++d) {
                  double* gp = outs + (rv + 1 + d) * S::threads + t;
                  const long long x = E == pg::fx::EXP_NONFINITE ? 0 : pg::fx::to_fixed(*gp, E, pg::fx::TOP_TERMS);
                  *reinterpret_cast<long long*>(gp) = x;
                }
              }
          __syncthreads();
        }
      }

      if (active) {
#pragma unroll
        for (int o = 0; o < pg::MAX_OUTS; ++o) {
          if (o < P.nout) {
            const OutDesc& od = P.outs[o];
            const bool has_v = flags & (1 << (2 * o));
            const bool has_g = flags & (2 << (2 * o));
            const int row0 = tab->out_row0[o];
            for (int c = 0; c < od.ncomp; ++c) {
              number r;
              if constexpr (FXC) {
                const int rv = row0 + c * (1 + dim);
                if (fx_int)
                  r = integrate_row_fx<dim, degree>(tab, outs, rv, has_v, has_g, t, lc, q, qa, qb, qc,
                                                    ex_out[rv * cpb + lc]);
                else
                  r = integrate_row<dim, degree, number>(tab, outs, rv, has_v, has_g, t, lc, q, qa, qb, qc);
              } else {
                r = integrate_row<dim, degree, number>(tab, outs, row0 + c * (1 + dim), has_v, has_g, t, lc, q, qa,
                                                       qb, qc);
              }
              if (has_v || has_g) {
                const long long idx = node + c * P.N;
                const int target = od.cmap ? od.cmap[idx] : (int)idx;
                if (target >= 0) atomicAdd(static_cast<number*>(od.acc) + target, r);
              }
            }
          }
        }
      }
    } else {
      // diagonal by unit probes: for each SRC slot (one per block field) and each cell node i
#pragma unroll 1
      for (int s = 0; s < P.nslots; ++s) {
        const SlotDesc& sd = P.slots[s];
        if (!sd.is_src) continue;
        int row = 0;
        for (int s2 = 0; s2 < s; ++s2) row += P.slots[s2].ncomp;
        const int o = sd.out_index;
        const OutDesc& od = P.outs[o];
        const int row0 = tab->out_row0[o];
        number mine[3] = {number(0), number(0), number(0)};
#pragma unroll 1
        for (int i = 0; i < nq; ++i) {
          // submit zero to every SRC slot, identity at node i of this one
          int rr = 0;
          for (int s2 = 0; s2 < P.nslots; ++s2) {
            if (P.slots[s2].is_src)
              for (int c = 0; c < P.slots[s2].ncomp; ++c)
                vals[(rr + c) * S::threads + t] = (s2 == s && q == i) ? number(1) : number(0);
            rr += P.slots[s2].ncomp;
          }
          if (t == 0) sflags = 0;
          for (int r = 0; r < P.nrows_out; ++r) outs[r * S::threads + t] = number(0);
          __syncthreads();
          pg::CellCtx<dim, degree, number> ctx;
          ctx.tab = tab;
          ctx.vals = vals;
          ctx.outs = outs;
          ctx.stride = S::threads;
          ctx.lc = lc;
          ctx.q = q;
          ctx.cell[0] = cx;
          ctx.cell[1] = cy;
          ctx.cell[2] = cz;
          ctx.err = P.err;
          ctx.submitted = 0;
          if (active) {
            FieldContainer<dim, degree, number> fc(ctx);
            const SimulationTimer timer = P.timer_dev ? *P.timer_dev : P.timer;
            pde.compute_lhs(fc, timer, P.block_id);
            if (ctx.submitted) atomicOr(&sflags, ctx.submitted);
          }
          __syncthreads();
          const int flags = sflags;
          if (active && q == i) {
            const bool has_v = flags & (1 << (2 * o));
            const bool has_g = flags & (2 << (2 * o));
            for (int c = 0; c < sd.ncomp; ++c)
              mine[c] = integrate_row<dim, degree, number>(tab, outs, row0 + c * (1 + dim), has_v, has_g, t, lc, q,
                                                           qa, qb, qc);
          }
          __syncthreads();
          (void)row;
        }
        if (active) {
          for (int c = 0; c < sd.ncomp; ++c) {
            const long long idx = node + c * P.N;
            const int target = od.cmap ? od.cmap[idx] : (int)idx;
            if (target >= 0) atomicAdd(static_cast<number*>(od.acc) + target, mine[c]);
          }
        }
      }
    }
  }
}

}  // namespace ppf

#pragma pop_macro("compute_lhs")
#pragma pop_macro("compute_rhs")
