// Matrix-free cell kernel: gather -> evaluate -> user callback per quadrature point ->
// integrate -> condensed scatter, for one solve block on a uniform hyper-rectangle mesh.
//
// Restates the per-cell work of MFOperator::compute_local_operator
// (src/solvers/mf_operator.cc:34-80) with FieldContainer::reinit_and_eval /
// integrate_and_distribute (include/prismspf/core/field_container.h:794-882) as one GPU
// kernel:
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
//     Dirichlet rows are dropped; contributions of neighbouring cells meet through FP64
//     atomicAdd into a zeroed accumulator (the finalize kernel applies invM and the
//     constraints).
#pragma once

#include <cuda_runtime.h>

#include <prismspf/core/field_container.h>

namespace ppf {

using prismspf::FieldContainer;
using prismspf::SimulationTimer;
namespace pg = prismspf::gpu;

struct SlotDesc {
  const double* ptr;  // component-major vector (ncomp * N)
  const int* cmap;    // constraint map, used when constrained_read
  int ncomp;
  int constrained_read;  // homogeneous constrained read (FEEvaluation::read_dof_values)
};

struct OutDesc {
  double* acc;       // accumulator (ncomp * N), zeroed before the launch
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
  const void* tables;  // device copy of CellTables<dim,degree>
  SimulationTimer timer;
  unsigned int block_id;
  int* err;
};

template <int dim, int degree>
struct CellShape {
  static constexpr int n = degree + 1;
  static constexpr int nq = pg::ipow(n, dim);
  static constexpr int cpb = (256 / nq) > 0 ? (256 / nq) : 1;  // cells per thread block
  static constexpr int threads = cpb * nq;
};

template <int dim, int degree>
__host__ __device__ inline size_t cell_smem_bytes(int nrows_in, int nrows_out) {
  using S = CellShape<dim, degree>;
  size_t tab = (sizeof(pg::CellTables<dim, degree>) + 15) / 16 * 16;
  return tab + sizeof(double) * (size_t)(nrows_in + nrows_out) * S::threads + 16;
}

template <class PDE, int dim, int degree, bool LHS>
__global__ void __launch_bounds__(CellShape<dim, degree>::threads)
    cell_kernel(const CellLaunch P, const PDE pde) {
  using S = CellShape<dim, degree>;
  using Tab = pg::CellTables<dim, degree>;
  constexpr int n = S::n, nq = S::nq, cpb = S::cpb, k = degree;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Tab* tab = reinterpret_cast<Tab*>(smem_raw);
  double* vals = reinterpret_cast<double*>(smem_raw + (sizeof(Tab) + 15) / 16 * 16);
  double* outs = vals + P.nrows_in * S::threads;
  __shared__ int sflags;

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
      cx = (int)(cell % P.nc[0]);
      if (dim > 1) cy = (int)((cell / P.nc[0]) % P.nc[1]);
      if (dim > 2) cz = (int)(cell / ((long long)P.nc[0] * P.nc[1]));
      node = ((long long)(k * cz + qc) * P.nn[1] + (k * cy + qb)) * P.nn[0] + (k * cx + qa);
    }
    __syncthreads();  // tables staged; previous tile's integrate finished with vals/outs/sflags
    if (t == 0) sflags = 0;

    // gather (read_dof_values_plain, or read_dof_values for constrained src)
    {
      int row = 0;
#pragma unroll
      for (int s = 0; s < pg::MAX_SLOTS; ++s) {
        if (s < P.nslots) {
          const SlotDesc& sd = P.slots[s];
          for (int c = 0; c < sd.ncomp; ++c) {
            double v = 0.0;
            if (active) {
              const long long idx = node + c * P.N;
              if (sd.constrained_read) {
                const int m = sd.cmap[idx];
                v = m >= 0 ? __ldg(sd.ptr + m) : 0.0;
              } else {
                v = __ldg(sd.ptr + idx);
              }
            }
            vals[(row + c) * S::threads + t] = v;
          }
          row += sd.ncomp;
        }
      }
      for (int r = 0; r < P.nrows_out; ++r) outs[r * S::threads + t] = 0.0;
    }
    __syncthreads();

    // user callback at this quadrature point
    pg::CellCtx<dim, degree> ctx;
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
      FieldContainer<dim, degree, double> fc(ctx);
      if constexpr (LHS) pde.compute_lhs(fc, P.timer, P.block_id);
      else pde.compute_rhs(fc, P.timer, P.block_id);
      if (ctx.submitted) atomicOr(&sflags, ctx.submitted);
    }
    __syncthreads();
    const int flags = sflags;

    // integrate + condensed scatter
    if (active) {
#pragma unroll
      for (int o = 0; o < pg::MAX_OUTS; ++o) {
        if (o < P.nout) {
          const OutDesc& od = P.outs[o];
          const bool has_v = flags & (1 << (2 * o));
          const bool has_g = flags & (2 << (2 * o));
          const int row0 = tab->out_row0[o];
          for (int c = 0; c < od.ncomp; ++c) {
            const int rv = row0 + c * (1 + dim);
            double r = has_v ? outs[rv * S::threads + t] : 0.0;
            if (has_g) {
#pragma unroll
              for (int d = 0; d < dim; ++d) {
                const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
                const int id = d == 0 ? qa : (d == 1 ? qb : qc);
                const double* g = outs + (rv + 1 + d) * S::threads + lc * nq + (q - id * sd);
                const double* Dt = tab->Dt[id];
#pragma unroll
                for (int j = 0; j < n; ++j) r = fma(Dt[j], g[j * sd], r);
              }
            }
            if (has_v || has_g) {
              const long long idx = node + c * P.N;
              const int target = od.cmap ? od.cmap[idx] : (int)idx;
              if (target >= 0) atomicAdd(od.acc + target, r);
            }
          }
        }
      }
    }
  }
}

}  // namespace ppf
