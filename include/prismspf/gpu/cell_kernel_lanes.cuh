// Lane kernel: the cell loop of an FP64 Q1/Q2 operator on cubic cells with every contraction in
// exact 64-bit integers, laid out so that one lane of a warp is one cell.
//
// The same per-cell work as cell_kernel (MFOperator::compute_local_operator,
// src/solvers/mf_operator.cc:34-80, with FieldContainer::reinit_and_eval /
// integrate_and_distribute, include/prismspf/core/field_container.h:794-882): gather ->
// user callback per quadrature point -> integrate -> condensed scatter. The layout and the
// arithmetic differ:
//   * a thread block owns a tile of 32 cells; lane l of every warp is cell l of the tile. Warp w
//     takes the w-th point of the cell's first dim-1 directions and each of its threads the n
//     points above it along the last direction (a line of its cell): point (w, j) is
//     q = w + j * n^(dim-1) (Q2 3-D: 9 warps, 3 points a thread). Rows of shared memory are
//     [point][cell], so every access is a contiguous warp row, a point's position on its lines
//     is uniform across the warp, and the per-cell block exponents are shared-memory atomics on
//     32 distinct words, one per thread and row;
//   * derivatives: exact integer line sums of the nodal values' fixed-point copies, rounded
//     once by to_double_fast (prismspf/gpu/fixed_point.cuh) with 1/h_d folded in;
//   * integration: the submitted value term (as h v) and gradient terms of a cell and output
//     component share one block exponent; every node's integral is the exact integer sum
//     2^vw(q) X(q) + sum_d 2^wo_d(q) L_d(q) (L_d the Gauss-Lobatto line integral of the
//     gradient terms along d, the last direction's taken from the thread's own points; 2^vw and
//     2^wo the integer quadrature weights) rounded once with the scale detJ / (h W^dim): no FP64
//     instruction outside the user's callback. On GB300 the FP64 pipe retires about two
//     operations per SM per clock and every FP64 conversion runs on it too, so the integer path
//     (issue slots) replaces 9-10 FP64 operations per point;
//   * four block barriers per tile: nodal values and exponents, fixed-point copies, submitted
//     terms and exponents, their fixed-point copies. The value-row exponents alternate between
//     two buffers so that clearing the next tile's needs no extra barrier;
//   * the cell tables and the flat row lists are kernel parameters (constant-bank loads); every
//     output component is integrated (rows the callback leaves stay zero), so no branch depends
//     on which terms were submitted; lanes past the last cell recompute the last cell and skip
//     its scatter.
// Accuracy: every derivative and every node's integral is one rounding of an exact sum of
// values quantised to 2^-58 (derivatives) or 2^-52 (integration) of the largest magnitude of
// their cell and row, as in the other integer-contraction kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

#include <prismspf/gpu/cell_kernel.cuh>

#pragma push_macro("compute_rhs")
#pragma push_macro("compute_lhs")
#undef compute_rhs
#undef compute_lhs

namespace ppf {

// Q1/Q2 on a lane kernel tile: lane l of every warp is cell l of a 32-cell tile; warp w holds
// the w-th point of the cell's first dim-1 directions, and its thread the n points above it
// along the last direction (a line of the cell): point (w, j) is q = w + j * cols.
template <int dim, int degree>
struct LaneShape {
  static constexpr int n = degree + 1;
  static constexpr int nq = pg::ipow(n, dim);
  static constexpr int cols = nq / n;  // warps per block
  static constexpr int threads = 32 * cols;
};
constexpr int LANE_CPT = 32;  // cells per tile

// fixed-point top of the integration: |X| <= 2^53 and |L_d| <= 8 * 2^53 keep the weighted sum
// below 2^53 (2^6 + 3 * 2^4 * 8) < 2^62
constexpr int LANE_TOP_TERMS = 52;

// An operator may ask for a register budget (`cell_lane_min_blocks`, resident blocks per SM);
// the default aims at about 48 registers a thread (Cahn-Hilliard Q2 3-D: 4 blocks of 288 threads
// at 46 registers measured 0.210 ms per launch against 0.218 ms for 5 blocks at 38 registers,
// which the shared memory would allow)
template <class PDE, int threads, class = void>
struct CellLaneMinBlocks {
  static constexpr int value = 65536 / (threads * 48) > 0 ? (65536 / (threads * 48) < 32 ? 65536 / (threads * 48) : 32) : 1;
};
template <class PDE, int threads>
struct CellLaneMinBlocks<PDE, threads, std::void_t<decltype(PDE::cell_lane_min_blocks)>> {
  static constexpr int value = PDE::cell_lane_min_blocks;
};

// shared memory of a tile: the double copies of the nv value rows, the fixed-point copies of the
// ng gradient rows, the submitted terms (nout components of 1 + dim rows), then the block
// exponents (two buffers of nrows_in rows, one of nout)
template <int dim, int degree>
__host__ __device__ constexpr size_t lane_smem_bytes(int nv, int ng, int nrows_in, int nout) {
  using S = LaneShape<dim, degree>;
  return (size_t)S::nq * LANE_CPT * 8 * (size_t)(nv + ng + nout * (1 + dim)) +
         4 * (size_t)LANE_CPT * (size_t)(2 * nrows_in + nout);
}

// Gauss-Lobatto line integral of the terms g at the line's node j (line_integral of
// fixed_point.cuh), with j uniform across a warp
template <int n>
__device__ __forceinline__ long long lane_line_integral(int j, long long g0, long long g1, long long g2) {
  if constexpr (n == 2) {
    const long long s = g0 + g1;
    return j == 0 ? -s : s;
  } else {
    const long long A = g2 - g0;
    if (j == 1) return A * -4;
    const long long B = g0 + g2 + g1 * 4;
    return j == 0 ? A * 2 - B : A * 2 + B;
  }
}

// The rows of one launch as flat lists (built on the host from the launch record): input rows
// (one per component of each dependency slot) and output components (one per component of each
// block field, with its value row and dim gradient rows).
constexpr int LANE_MAX_IN = 6;
constexpr int LANE_MAX_OUT = 3;
struct LaneRows {
  int nin;
  int nout;
  int nv;                                // input rows with a double copy (read as values or Hessians)
  int ng;                                // input rows with a fixed-point copy (read as gradients)
  unsigned int div_m[2], div_l[2];       // cell index -> (x, y, z): multiply-high divisors of nc[0], nc[1]
  const double* in_base[LANE_MAX_IN];    // vector of the row's slot
  const int* in_cmap[LANE_MAX_IN];       // constraint map for a constrained read, else null
  unsigned int in_off[LANE_MAX_IN];      // component offset c * N
  double* out_acc[LANE_MAX_OUT];         // accumulator of the output's field
  const int* out_cmap[LANE_MAX_OUT];     // condensation map, else null
  unsigned int out_off[LANE_MAX_OUT];    // component offset c * N
  int out_row[LANE_MAX_OUT];             // value row of the component (dim gradient rows follow)
};

template <class PDE, int dim, int degree, int MODE, int MINB>
__global__ void __launch_bounds__(LaneShape<dim, degree>::threads, MINB)
    cell_kernel_lanes(const __grid_constant__ CellLaunch P, const __grid_constant__ PDE pde,
                      const __grid_constant__ pg::CellTables<dim, degree, double> T,
                      const __grid_constant__ LaneRows R) {
  static_assert(degree <= 2 && MODE != MODE_DIAG, "the lane kernel covers FP64 Q1/Q2 RHS and LHS launches");
  using S = LaneShape<dim, degree>;
  using Tab = pg::CellTables<dim, degree, double>;
  namespace fx = pg::fx;
  constexpr int n = S::n, nq = S::nq, cols = S::cols, k = degree, CPT = LANE_CPT;
  constexpr int ROW = nq * CPT;   // entries of one row
  constexpr int JS = cols * CPT;  // entry stride between a thread's points
  constexpr int TOPT = LANE_TOP_TERMS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the tables are a kernel parameter: read-only constant-bank loads, uniform where their index is
  const Tab* tab = &T;
  double* vals = reinterpret_cast<double*>(smem_raw);               // [nv][q][cell]
  long long* vfx = reinterpret_cast<long long*>(vals + R.nv * ROW);  // [ng][q][cell]
  double* outs = reinterpret_cast<double*>(vfx + R.ng * ROW);       // [out rows][q][cell]
  const int nrows_out = R.nout * (1 + dim);
  int* ex_in = reinterpret_cast<int*>(outs + nrows_out * ROW);       // [2][nin][cell]
  int* ex_out = ex_in + 2 * R.nin * CPT;                             // [nout][cell]

  const int t = threadIdx.x;
  const int lc = t & 31;
  const int w = t >> 5;          // point of the first dim-1 directions
  const int p0 = w * CPT + lc;   // entry of the thread's first point; point j at p0 + j * JS
  const int qa = w % n;
  const int qb = dim > 2 ? w / n : 0;
  const unsigned int fx_rows = tab->fx_rows;  // input rows read as gradients (fixed-point copies)
  const int hpow2 = tab->hpow2, hk = tab->hk;
  const unsigned long long hsig = tab->hsig;
  // both exponent buffers: 0 for rows with a fixed-point copy, -1 for rows read as values only
  for (int i = t; i < 2 * R.nin * CPT; i += S::threads) ex_in[i] = ((fx_rows >> ((i / CPT) % R.nin)) & 1u) ? 0 : -1;
  const unsigned int nn0 = (unsigned int)P.nn[0], nn1 = (unsigned int)P.nn[1];
  const unsigned int lstride = dim > 2 ? nn0 * nn1 : nn0;  // lattice stride of the last direction
  const unsigned int ncells = (unsigned int)P.ncells;
  const unsigned int ntiles = (ncells + CPT - 1) / CPT;
  __syncthreads();  // exponent buffers set

  int par = 0;
  for (unsigned int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, par ^= 1) {
    int* exi = ex_in + par * R.nin * CPT;
    int* exn = ex_in + (par ^ 1) * R.nin * CPT;
    // lanes past the last cell redo the last cell and skip its scatter
    const unsigned int cell_t = tile * CPT + lc;
    const bool active = cell_t < ncells;
    const unsigned int cell = active ? cell_t : ncells - 1;
    int cx, cy = 0, cz = 0;
    {
      const unsigned int q0 = (__umulhi(cell, R.div_m[0]) + cell) >> R.div_l[0];
      cx = (int)(cell - q0 * (unsigned int)P.nc[0]);
      if (dim == 2) cy = (int)q0;
      if (dim > 2) {
        const unsigned int q1 = (__umulhi(q0, R.div_m[1]) + q0) >> R.div_l[1];
        cy = (int)(q0 - q1 * (unsigned int)P.nc[1]);
        cz = (int)q1;
      }
    }
    // lattice node of the thread's first point (last-direction index 0)
    const unsigned int node0 = dim > 2 ? ((unsigned int)(k * cz) * nn1 + (unsigned int)(k * cy + qb)) * nn0 + (unsigned int)(k * cx + qa)
                                       : (unsigned int)(k * cy) * nn0 + (unsigned int)(k * cx + qa);

    // gather (read_dof_values_plain, or read_dof_values for a constrained src) and the block
    // exponents of the rows read as gradients
#pragma unroll
    for (int r = 0; r < LANE_MAX_IN; ++r) {
      if (r < R.nin) {
        const double* base = R.in_base[r];
        int e = 0;
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const unsigned int idx = node0 + (unsigned int)j * lstride + R.in_off[r];
          double v;
          if (R.in_cmap[r]) {
            const int m = __ldg(R.in_cmap[r] + idx);
            const double own = __ldg(base + idx);
            v = m == (int)idx ? own : (m >= 0 ? __ldg(base + m) : 0.0);
          } else {
            v = __ldg(base + idx);
          }
          const int vs = tab->lane_vslot[r], gs = tab->lane_gslot[r];
          if (vs >= 0) vals[vs * ROW + p0 + j * JS] = v;
          // a gradient row's double stays in its fixed-point slot until converted in place
          if (gs >= 0) vfx[gs * ROW + p0 + j * JS] = __double_as_longlong(v);
          e = max(e, fx::exponent(v));
        }
        if ((fx_rows >> r) & 1u) atomicMax(&exi[r * CPT + lc], e);
      }
    }
    __syncthreads();  // nodal values and their block exponents complete

    // fixed-point copies; clear the submitted terms, their exponents and the next tile's
    // value-row exponents
#pragma unroll
    for (int r = 0; r < LANE_MAX_IN; ++r) {
      if (r < R.nin && ((fx_rows >> r) & 1u)) {
        // (a cell holding a non-finite value gets meaningless copies: every result read from them
        // is replaced by NaN)
        const int E = exi[r * CPT + lc];
        long long* x = vfx + tab->lane_gslot[r] * ROW + p0;
#pragma unroll
        for (int j = 0; j < n; ++j) x[j * JS] = fx::to_fixed_fast<fx::TOP_VALUES>(__longlong_as_double(x[j * JS]), E);
      }
    }
#pragma unroll
    for (int o = 0; o < LANE_MAX_OUT; ++o)
      if (o < R.nout)
#pragma unroll
        for (int i = 0; i <= dim; ++i)
#pragma unroll
          for (int j = 0; j < n; ++j) outs[(R.out_row[o] + i) * ROW + p0 + j * JS] = 0.0;
    for (int i = t; i < R.nin * CPT; i += S::threads) exn[i] = ((fx_rows >> (i / CPT)) & 1u) ? 0 : -1;
    for (int i = t; i < R.nout * CPT; i += S::threads) ex_out[i] = 0;
    __syncthreads();  // fixed-point copies visible

    // the user callback at each of the thread's points
    const SimulationTimer& timer = P.timer_dev ? *P.timer_dev : P.timer;
    // (one copy of the callback's code: unrolling the points measured slower)
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
      pg::CellCtx<dim, degree, double> ctx;
      ctx.tab = tab;
      ctx.vals = vals;
      ctx.outs = outs;
      ctx.stride = ROW;
      ctx.lc = lc;
      ctx.q = w + j * cols;
      ctx.cell[0] = cx;
      ctx.cell[1] = cy;
      ctx.cell[2] = cz;
      ctx.err = P.err;
      ctx.submitted = 0;
      ctx.vals_fx = vfx;
      ctx.ex_in = exi;
      ctx.cpb = CPT;
      ctx.cpt = CPT;
      ctx.lean = 1;
      ctx.qi[0] = qa;
      ctx.qi[1] = dim > 2 ? qb : j;
      ctx.qi[2] = dim > 2 ? j : 0;
      FieldContainer<dim, degree, double> fc(ctx);
      if constexpr (MODE == MODE_LHS) pde.compute_lhs(fc, timer, P.block_id);
      else pde.compute_rhs(fc, timer, P.block_id);
    }
    // block exponents of every output component's terms (rows the callback left are zero): the
    // value term enters as h v (one binade more when h is not a power of two)
#pragma unroll
    for (int o = 0; o < LANE_MAX_OUT; ++o) {
      if (o < R.nout) {
        const int rv = R.out_row[o];
        int e = 0;
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const int ev = fx::exponent(outs[rv * ROW + p0 + j * JS]);
          const int eh = ev + hk + (hpow2 ? 0 : 1);
          e = max(e, ev == 0 ? 0 : (ev == fx::EXP_NONFINITE || eh >= fx::EXP_NONFINITE ? fx::EXP_NONFINITE : max(eh, 0)));
#pragma unroll
          for (int d = 0; d < dim; ++d) e = max(e, fx::exponent(outs[(rv + 1 + d) * ROW + p0 + j * JS]));
        }
        atomicMax(&ex_out[o * CPT + lc], e);
      }
    }
    __syncthreads();  // submitted terms and their block exponents complete

    // the submitted terms in place to fixed point
#pragma unroll
    for (int o = 0; o < LANE_MAX_OUT; ++o) {
      if (o < R.nout) {
        const int rv = R.out_row[o];
        // (with E = 2047 the copies are meaningless and the integral is replaced by NaN)
        const int E = ex_out[o * CPT + lc];
        long long* ox = reinterpret_cast<long long*>(outs);
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const int e0 = rv * ROW + p0 + j * JS;
          const double v = outs[e0];
          ox[e0] = hpow2 ? fx::to_fixed_fast<TOPT>(v, E - hk) : fx::to_fixed_scaled<TOPT>(v, E, hsig, hk);
#pragma unroll
          for (int d = 0; d < dim; ++d) ox[e0 + (1 + d) * ROW] = fx::to_fixed_fast<TOPT>(outs[e0 + (1 + d) * ROW], E);
        }
      }
    }
    __syncthreads();  // fixed-point terms visible

    // integrate and scatter (distribute_local_to_global through the constraint map)
    const long long* ox = reinterpret_cast<const long long*>(outs);
#pragma unroll
    for (int o = 0; o < LANE_MAX_OUT; ++o) {
      if (o < R.nout) {
        const int rv = R.out_row[o];
        const int E = ex_out[o * CPT + lc];
        // the last direction's line is the thread's own points
        const long long* gl = ox + (rv + dim) * ROW + p0;
        const long long z0 = gl[0], z1 = gl[JS], z2 = n > 2 ? gl[2 * JS] : 0ll;
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const int q = w + j * cols;
          const int e0 = rv * ROW + p0 + j * JS;
          // this point's integration weights: powers of two from the tables
          long long Tx = (long long)((unsigned long long)ox[e0] << tab->vw_sh[q]);
#pragma unroll
          for (int d = 0; d < dim - 1; ++d) {
            const int sd = d == 0 ? 1 : n;
            const int id = d == 0 ? qa : qb;
            const long long* g = ox + (rv + 1 + d) * ROW + (q - id * sd) * CPT + lc;
            const long long L = lane_line_integral<n>(id, g[0], g[sd * CPT], n > 2 ? g[2 * sd * CPT] : 0ll);
            Tx += (long long)((unsigned long long)L << tab->wo_sh[d][q]);
          }
          const long long Lz = lane_line_integral<n>(j, z0, z1, z2);
          Tx += (long long)((unsigned long long)Lz << tab->wo_sh[dim - 1][q]);
          const double rr = fx::to_double_fast(Tx, E - 1023 - TOPT + tab->ik[0], tab->isig[0], true);
          const double r = E == fx::EXP_NONFINITE ? fx::quiet_nan() : rr;
          const unsigned int idx = node0 + (unsigned int)j * lstride + R.out_off[o];
          const int target = R.out_cmap[o] ? __ldg(R.out_cmap[o] + idx) : (int)idx;
          if (active && target >= 0) atomicAdd(R.out_acc[o] + target, r);
        }
      }
    }
  }
}

// FP32 operators (the smoothing levels of a mixed-precision V-cycle) on the same layout: 32 cells
// a tile, a line of each cell per thread, plain FP32 contractions (derivatives from the nodal
// values, integration with the tables' jdt weights), so a tile needs two barriers (nodal values;
// submitted terms). Any cell shape.
template <int dim, int degree>
__host__ __device__ constexpr size_t lane_f32_smem_bytes(int nrows_in, int nrows_out) {
  using S = LaneShape<dim, degree>;
  return (size_t)S::nq * LANE_CPT * 4 * (size_t)(nrows_in + nrows_out);
}

template <class PDE, int dim, int degree, int MODE, int MINB>
__global__ void __launch_bounds__(LaneShape<dim, degree>::threads, MINB)
    cell_kernel_lanes_f32(const __grid_constant__ CellLaunch P, const __grid_constant__ PDE pde,
                          const __grid_constant__ pg::CellTables<dim, degree, float> T,
                          const __grid_constant__ LaneRows R) {
  static_assert(degree <= 2 && MODE == MODE_LHS, "the FP32 lane kernel covers Q1/Q2 LHS launches");
  using S = LaneShape<dim, degree>;
  using Tab = pg::CellTables<dim, degree, float>;
  constexpr int n = S::n, nq = S::nq, cols = S::cols, k = degree, CPT = LANE_CPT;
  constexpr int ROW = nq * CPT;
  constexpr int JS = cols * CPT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Tab* tab = &T;
  float* vals = reinterpret_cast<float*>(smem_raw);  // [nin][q][cell]
  float* outs = vals + R.nin * ROW;                  // [out rows][q][cell]
  const int t = threadIdx.x;
  const int lc = t & 31;
  const int w = t >> 5;
  const int p0 = w * CPT + lc;
  const int qa = w % n;
  const int qb = dim > 2 ? w / n : 0;
  const unsigned int nn0 = (unsigned int)P.nn[0], nn1 = (unsigned int)P.nn[1];
  const unsigned int lstride = dim > 2 ? nn0 * nn1 : nn0;
  const unsigned int ncells = (unsigned int)P.ncells;
  const unsigned int ntiles = (ncells + CPT - 1) / CPT;

  for (unsigned int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const unsigned int cell_t = tile * CPT + lc;
    const bool active = cell_t < ncells;
    const unsigned int cell = active ? cell_t : ncells - 1;
    int cx, cy = 0, cz = 0;
    {
      const unsigned int q0 = (__umulhi(cell, R.div_m[0]) + cell) >> R.div_l[0];
      cx = (int)(cell - q0 * (unsigned int)P.nc[0]);
      if (dim == 2) cy = (int)q0;
      if (dim > 2) {
        const unsigned int q1 = (__umulhi(q0, R.div_m[1]) + q0) >> R.div_l[1];
        cy = (int)(q0 - q1 * (unsigned int)P.nc[1]);
        cz = (int)q1;
      }
    }
    const unsigned int node0 = dim > 2 ? ((unsigned int)(k * cz) * nn1 + (unsigned int)(k * cy + qb)) * nn0 + (unsigned int)(k * cx + qa)
                                       : (unsigned int)(k * cy) * nn0 + (unsigned int)(k * cx + qa);
    // the previous tile's integration read the submitted terms and values: done by all threads
    __syncthreads();
#pragma unroll
    for (int r = 0; r < LANE_MAX_IN; ++r) {
      if (r < R.nin) {
        const float* base = reinterpret_cast<const float*>(R.in_base[r]);
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const unsigned int idx = node0 + (unsigned int)j * lstride + R.in_off[r];
          float v;
          if (R.in_cmap[r]) {
            const int m = __ldg(R.in_cmap[r] + idx);
            const float own = __ldg(base + idx);
            v = m == (int)idx ? own : (m >= 0 ? __ldg(base + m) : 0.f);
          } else {
            v = __ldg(base + idx);
          }
          vals[r * ROW + p0 + j * JS] = v;
        }
      }
    }
#pragma unroll
    for (int o = 0; o < LANE_MAX_OUT; ++o)
      if (o < R.nout)
#pragma unroll
        for (int i = 0; i <= dim; ++i)
#pragma unroll
          for (int j = 0; j < n; ++j) outs[(R.out_row[o] + i) * ROW + p0 + j * JS] = 0.f;
    __syncthreads();  // nodal values visible

    const SimulationTimer& timer = P.timer_dev ? *P.timer_dev : P.timer;
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
      pg::CellCtx<dim, degree, float> ctx;
      ctx.tab = tab;
      ctx.vals = vals;
      ctx.outs = outs;
      ctx.stride = ROW;
      ctx.lc = lc;
      ctx.q = w + j * cols;
      ctx.cell[0] = cx;
      ctx.cell[1] = cy;
      ctx.cell[2] = cz;
      ctx.err = P.err;
      ctx.submitted = 0;
      ctx.cpt = CPT;
      FieldContainer<dim, degree, float> fc(ctx);
      pde.compute_lhs(fc, timer, P.block_id);
    }
    __syncthreads();  // submitted terms visible

    // integrate (the tables' jdt weights) and scatter
#pragma unroll
    for (int o = 0; o < LANE_MAX_OUT; ++o) {
      if (o < R.nout) {
        const int rv = R.out_row[o];
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const int q = w + j * cols;
          const int qi[3] = {qa, dim > 2 ? qb : j, dim > 2 ? j : 0};
          float r = outs[rv * ROW + p0 + j * JS];
#pragma unroll
          for (int d = 0; d < dim; ++d) {
            const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
            const float* g = outs + (rv + 1 + d) * ROW + (q - qi[d] * sd) * CPT + lc;
            const float* wt = tab->jdt[d][q];
#pragma unroll
            for (int m = 0; m < n; ++m) r = fmaf(wt[m], g[m * sd * CPT], r);
          }
          const unsigned int idx = node0 + (unsigned int)j * lstride + R.out_off[o];
          const int target = R.out_cmap[o] ? __ldg(R.out_cmap[o] + idx) : (int)idx;
          if (active && target >= 0) atomicAdd(reinterpret_cast<float*>(R.out_acc[o]) + target, r);
        }
      }
    }
  }
}

// the flat row lists of a launch record; false when they exceed the lane kernel's limits
inline bool lane_rows(const CellLaunch& P, int dim, LaneRows* R) {
  std::memset(R, 0, sizeof(*R));
  int r = 0;
  for (int s = 0; s < P.nslots; ++s) {
    const SlotDesc& sd = P.slots[s];
    for (int c = 0; c < sd.ncomp; ++c, ++r) {
      if (r >= LANE_MAX_IN) return false;
      R->in_base[r] = static_cast<const double*>(sd.ptr);
      R->in_cmap[r] = sd.constrained_read ? sd.cmap : nullptr;
      R->in_off[r] = (unsigned int)(c * P.N);
    }
  }
  R->nin = r;
  if (r != P.nrows_in) return false;
  int o = 0, row = 0;
  for (int i = 0; i < P.nout; ++i) {
    const OutDesc& od = P.outs[i];
    for (int c = 0; c < od.ncomp; ++c, ++o) {
      if (o >= LANE_MAX_OUT) return false;
      R->out_acc[o] = static_cast<double*>(od.acc);
      R->out_cmap[o] = od.cmap;
      R->out_off[o] = (unsigned int)(c * P.N);
      R->out_row[o] = row;
      row += 1 + dim;
    }
  }
  R->nout = o;
  for (int d = 0; d < 2; ++d) {
    pg::fx::FastDiv f;
    f.init((unsigned int)P.nc[d]);
    R->div_m[d] = f.m;
    R->div_l[d] = f.l;
  }
  return row == P.nrows_out;
}

template <class PDE, int dim, int degree, int mode, int MINB>
cudaError_t launch_lanes(const CellLaunch& P, const LaneRows& R, const void* obj, cudaStream_t s) {
  using S = LaneShape<dim, degree>;
  auto kern = cell_kernel_lanes<PDE, dim, degree, mode, MINB>;
  const size_t smem = lane_smem_bytes<dim, degree>(R.nv, R.ng, R.nin, R.nout);
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
  const long long ntiles = (P.ncells + LANE_CPT - 1) / LANE_CPT;
  long long grid = (long long)sms * occ;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, S::threads, smem, s>>>(P, *reinterpret_cast<const PDE*>(obj),
                                                *reinterpret_cast<const pg::CellTables<dim, degree, double>*>(P.tables_host),
                                                R);
  return cudaGetLastError();
}

template <class PDE, int dim, int degree, int MINB>
cudaError_t launch_lanes_f32(const CellLaunch& P, const LaneRows& R, const void* obj, cudaStream_t s) {
  using S = LaneShape<dim, degree>;
  auto kern = cell_kernel_lanes_f32<PDE, dim, degree, MODE_LHS, MINB>;
  const size_t smem = lane_f32_smem_bytes<dim, degree>(R.nin, P.nrows_out);
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
  const long long ntiles = (P.ncells + LANE_CPT - 1) / LANE_CPT;
  long long grid = (long long)sms * occ;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, S::threads, smem, s>>>(P, *reinterpret_cast<const PDE*>(obj),
                                                *reinterpret_cast<const pg::CellTables<dim, degree, float>*>(P.tables_host),
                                                R);
  return cudaGetLastError();
}

// the FP32 lane kernel for an FP32 Q1/Q2 left-hand side, or cudaErrorNotSupported
template <class PDE, int dim, int degree>
cudaError_t launch_cell_kernel_lanes_f32_impl(const CellLaunch& P, const void* obj, cudaStream_t s) {
  constexpr int MINB = CellLaneMinBlocks<PDE, LaneShape<dim, degree>::threads>::value;
  LaneRows R;
  if (!P.tables_host || !lane_rows(P, dim, &R)) return cudaErrorNotSupported;
  if (lane_f32_smem_bytes<dim, degree>(R.nin, P.nrows_out) > 232448) return cudaErrorNotSupported;
  return launch_lanes_f32<PDE, dim, degree, MINB>(P, R, obj, s);
}

// launches the lane kernel, or returns cudaErrorNotSupported when the launch's rows exceed its
// limits (the caller then takes the thread-block kernel)
template <class PDE, int dim, int degree, int mode>
cudaError_t launch_cell_kernel_lanes_impl(const CellLaunch& P, const void* obj, cudaStream_t s) {
  constexpr int MINB = CellLaneMinBlocks<PDE, LaneShape<dim, degree>::threads>::value;
  LaneRows R;
  if (!P.tables_host || !lane_rows(P, dim, &R)) return cudaErrorNotSupported;
  const auto* tab = static_cast<const pg::CellTables<dim, degree, double>*>(P.tables_host);
  const unsigned int mask = (1u << R.nin) - 1u;
  R.nv = __builtin_popcount(tab->val_rows & mask);
  R.ng = __builtin_popcount(tab->fx_rows & mask);
  if (lane_smem_bytes<dim, degree>(R.nv, R.ng, R.nin, R.nout) > 232448) return cudaErrorNotSupported;
  return launch_lanes<PDE, dim, degree, mode, MINB>(P, R, obj, s);
}

}  // namespace ppf

#pragma pop_macro("compute_lhs")
#pragma pop_macro("compute_rhs")
