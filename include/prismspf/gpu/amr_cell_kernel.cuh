// Matrix-free cell kernel on an adaptive (hanging-node) mesh: the work of
// MFOperator::compute_local_operator (src/solvers/mf_operator.cc:34-80) for the active cells of
// a forest of quadtrees / octrees, one thread per (cell, quadrature point) as in cell_kernel:
//   * cells are a list (level, integer coordinates at that level) with an explicit table of
//     their (degree+1)^dim DoF indices (lexicographic nodes), since neighbouring cells may
//     differ by one level;
//   * the per-launch CellTables are staged for every level in use: cells of level l read the
//     metric terms of a cell of size size / (subdivisions 2^l), so FieldContainer and the user
//     operator see exactly what they see on a uniform mesh of that level;
//   * constraint maps per component: cmap[i] = i (free), -1-j (Dirichlet row j), or
//     AMR_HANG_BASE + r (hanging row r: u_i = sum_e w_e u_{master_e}, masters free or
//     Dirichlet). read_dof_values (constrained src) interpolates hanging entries with Dirichlet
//     masters read as zero; distribute_local_to_global adds a hanging row's contribution
//     w_e r to its free masters and drops Dirichlet rows.
#pragma once

#include <prismspf/gpu/cell_kernel.cuh>

#pragma push_macro("compute_rhs")
#pragma push_macro("compute_lhs")
#undef compute_rhs
#undef compute_lhs

namespace ppf {

constexpr int MODE_AMR = 8;             // mode flag: the launch record is an AmrCellLaunch
constexpr int AMR_HANG_BASE = 1 << 30;  // cmap entries from here on name a hanging row

struct AmrCellLaunch {
  CellLaunch base;        // base.tables: nlev consecutive CellTables, the coarsest level first
  const int* cell_dofs;   // ncells * (degree+1)^dim DoF indices
  const int4* cell_info;  // per cell: level - coarsest level, x, y, z (coordinates at that level)
  int nlev;
  const int* h_ptr;       // hanging rows: masters h_idx[h_ptr[r] .. h_ptr[r+1]) with weights h_w
  const int* h_idx;
  const double* h_w;
};

template <int dim, int degree, typename number>
__host__ __device__ inline size_t amr_cell_smem_bytes(int nlev, int nrows_in, int nrows_out) {
  using S = CellShape<dim, degree>;
  const size_t tab = (sizeof(pg::CellTables<dim, degree, number>) + 15) / 16 * 16;
  size_t b = tab * (size_t)nlev + sizeof(number) * (size_t)(nrows_in + nrows_out) * S::threads + 16;
  // integer derivatives (FP64 Q1/Q2): fixed-point values and per-cell block exponents
  if (cell_fx_capable<dim, degree, number>())
    b += sizeof(long long) * (size_t)nrows_in * S::threads + sizeof(int) * (size_t)nrows_in * S::cpb;
  return b;
}

template <class PDE, int dim, int degree, int MODE, typename number>
__global__ void __launch_bounds__(CellShape<dim, degree>::threads, 1)
    amr_cell_kernel(const __grid_constant__ AmrCellLaunch A, const __grid_constant__ PDE pde) {
  static_assert(MODE == MODE_RHS || MODE == MODE_LHS, "adaptive meshes evaluate rhs and lhs operators");
  using S = CellShape<dim, degree>;
  using Tab = pg::CellTables<dim, degree, number>;
  constexpr int n = S::n, nq = S::nq, cpb = S::cpb;
  constexpr size_t tab_stride = (sizeof(Tab) + 15) / 16 * 16;
  const CellLaunch& P = A.base;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  number* vals = reinterpret_cast<number*>(smem_raw + tab_stride * A.nlev);
  number* outs = vals + P.nrows_in * S::threads;
  __shared__ int sflags;
  // integer derivatives (fixed_point.cuh) with every level's tables, FP64 integration
  constexpr bool FXC = cell_fx_capable<dim, degree, number>();
  long long* vals_fx = reinterpret_cast<long long*>(outs + P.nrows_out * S::threads);
  int* ex_in = reinterpret_cast<int*>(vals_fx + P.nrows_in * S::threads);
  bool fx_on = false;
  unsigned int fx_rows = 0;
  if constexpr (FXC) {
    unsigned int dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const Tab* g0 = static_cast<const Tab*>(P.tables);
    fx_on = P.fx_deriv != 0 && g0->fx != 0 &&
            dyn >= (unsigned int)amr_cell_smem_bytes<dim, degree, number>(A.nlev, P.nrows_in, P.nrows_out);
    fx_rows = g0->fx_rows;
  }

  for (int l = 0; l < A.nlev; ++l) {
    const int nwords = (int)(sizeof(Tab) / 4);
    const unsigned int* src =
        reinterpret_cast<const unsigned int*>(static_cast<const unsigned char*>(P.tables) + sizeof(Tab) * l);
    unsigned int* dst = reinterpret_cast<unsigned int*>(smem_raw + tab_stride * l);
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
  }
  const Tab* tab0 = reinterpret_cast<const Tab*>(smem_raw);

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
    int4 info = make_int4(0, 0, 0, 0);
    long long dof = 0;
    if (active) {
      info = __ldg(A.cell_info + cell);
      dof = __ldg(A.cell_dofs + cell * nq + q);
    }
    if constexpr (FXC) {
      // last read by the previous tile's callbacks; rows without a fixed-point copy keep -1
      if (fx_on)
        for (int i = t; i < P.nrows_in * cpb; i += S::threads) ex_in[i] = ((fx_rows >> (i / cpb)) & 1u) ? 0 : -1;
    }
    __syncthreads();  // tables staged; previous tile finished with vals/outs/sflags

    {
      int row = 0;
#pragma unroll
      for (int s = 0; s < pg::MAX_SLOTS; ++s) {
        if (s < P.nslots) {
          const SlotDesc& sd = P.slots[s];
          const number* ptr = static_cast<const number*>(sd.ptr);
          for (int c = 0; c < sd.ncomp; ++c) {
            number v = number(0);
            if (active) {
              const long long base = c * P.N;
              const long long idx = dof + base;
              if (sd.constrained_read) {
                const int m = __ldg(sd.cmap + idx);
                if (m == (int)idx) {
                  v = __ldg(ptr + idx);
                } else if (m >= AMR_HANG_BASE) {
                  const int r = m - AMR_HANG_BASE;
                  for (int e = __ldg(A.h_ptr + r); e < __ldg(A.h_ptr + r + 1); ++e) {
                    const long long mi = base + __ldg(A.h_idx + e);
                    if (__ldg(sd.cmap + mi) == (int)mi) v += number(__ldg(A.h_w + e)) * __ldg(ptr + mi);
                  }
                }
              } else {
                v = __ldg(ptr + idx);
              }
            }
            vals[(row + c) * S::threads + t] = v;
            if constexpr (FXC) {
              if (fx_on && ((fx_rows >> (row + c)) & 1u)) atomicMax(&ex_in[(row + c) * cpb + lc], pg::fx::exponent(v));
            }
          }
          row += sd.ncomp;
        }
      }
    }

    if constexpr (FXC) {
      if (fx_on) {
        __syncthreads();  // block exponents of the value rows complete
        for (int r = 0; r < P.nrows_in; ++r) {
          const int E = ex_in[r * cpb + lc];
          if (E >= 0 && E != pg::fx::EXP_NONFINITE)
            vals_fx[r * S::threads + t] = pg::fx::to_fixed(vals[r * S::threads + t], E, pg::fx::TOP_VALUES);
        }
      }
    }
    if (t == 0) sflags = 0;
    for (int r = 0; r < P.nrows_out; ++r) outs[r * S::threads + t] = number(0);
    __syncthreads();

    pg::CellCtx<dim, degree, number> ctx;
    ctx.tab = reinterpret_cast<const Tab*>(smem_raw + tab_stride * info.x);
    if constexpr (FXC) {
      if (fx_on) {
        ctx.vals_fx = vals_fx;
        ctx.ex_in = ex_in;
        ctx.cpb = cpb;
      }
    }
    ctx.vals = vals;
    ctx.outs = outs;
    ctx.stride = S::threads;
    ctx.lc = lc;
    ctx.q = q;
    ctx.cell[0] = info.y;
    ctx.cell[1] = info.z;
    ctx.cell[2] = info.w;
    ctx.err = P.err;
    ctx.submitted = 0;
    if (active) {
      FieldContainer<dim, degree, number> fc(ctx);
      const SimulationTimer timer = P.timer_dev ? *P.timer_dev : P.timer;
      if constexpr (MODE == MODE_LHS) pde.compute_lhs(fc, timer, P.block_id);
      else pde.compute_rhs(fc, timer, P.block_id);
      if (ctx.submitted) atomicOr(&sflags, ctx.submitted);
    }
    __syncthreads();
    const int flags = sflags;

    if (active) {
#pragma unroll
      for (int o = 0; o < pg::MAX_OUTS; ++o) {
        if (o < P.nout) {
          const OutDesc& od = P.outs[o];
          const bool has_v = flags & (1 << (2 * o));
          const bool has_g = flags & (2 << (2 * o));
          const int row0 = tab0->out_row0[o];
          for (int c = 0; c < od.ncomp; ++c) {
            // the integration weights are the cell's level's
            const number r = integrate_row<dim, degree, number>(ctx.tab, outs, row0 + c * (1 + dim), has_v, has_g,
                                                                t, lc, q, qa, qb, qc);
            if (!(has_v || has_g)) continue;
            const long long base = c * P.N;
            const long long idx = dof + base;
            number* acc = static_cast<number*>(od.acc);
            const int target = od.cmap ? od.cmap[idx] : (int)idx;
            if (target >= AMR_HANG_BASE) {
              const int hr = target - AMR_HANG_BASE;
              for (int e = __ldg(A.h_ptr + hr); e < __ldg(A.h_ptr + hr + 1); ++e) {
                const long long mi = base + __ldg(A.h_idx + e);
                if (od.cmap[mi] == (int)mi) atomicAdd(acc + mi, number(__ldg(A.h_w + e)) * r);
              }
            } else if (target >= 0) {
              atomicAdd(acc + target, r);
            }
          }
        }
      }
    }
  }
}

template <class PDE, int dim, int degree, int mode, typename number>
cudaError_t launch_amr_cell_kernel(const AmrCellLaunch& A, const void* obj, size_t smem, cudaStream_t s) {
  using S = CellShape<dim, degree>;
  auto kern = amr_cell_kernel<PDE, dim, degree, mode, number>;
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
  const long long ntiles = (A.base.ncells + S::cpb - 1) / S::cpb;
  long long grid = (long long)sms * occ;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, S::threads, smem, s>>>(A, *reinterpret_cast<const PDE*>(obj));
  return cudaGetLastError();
}

}  // namespace ppf

#pragma pop_macro("compute_lhs")
#pragma pop_macro("compute_rhs")
