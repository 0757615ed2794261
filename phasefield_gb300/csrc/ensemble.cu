// Batched ensemble of independent explicit Allen-Cahn simulations (block 1 of
// applications/allen_cahn/explicit) of uneven mesh size, degree (Q1/Q2) and parameters,
// advanced by ONE kernel launch per time step, the step loop captured in a CUDA graph.
//
// GB300 design:
//   * no grid-wide barrier: the state of each instance is kept as its un-normalised
//     accumulator; a step reads the accumulator of step k, forms n = invM (.) acc on the fly
//     in the gather (the same product the single-simulation finalize kernel computes), and
//     scatters the cell integrals of step k+1 into a second accumulator, while it zeroes a
//     third one (read one step earlier, so no block of this launch touches it). The three
//     accumulators rotate; a launch depends only on the previous launch having finished.
//   * one persistent launch for every instance and both degrees: a global list of cell tiles
//     (instance, first cell) is walked grid-stride; a tile of a Q1 instance runs the Q1 body,
//     of a Q2 instance the Q2 body (block-uniform branch), with the instance's parameters
//     (m_well, kappa) and its cell tables, built once on the host with the engine's table
//     builder for the instance's mesh spacing, copied into shared memory per tile (an integer
//     copy: GB300's FP64 pipe is too narrow to recompute them per tile).
//   * tile shapes (cells per tile for Q1 and for Q2) and the grid size are chosen by a
//     project-written autotuner that times candidate shapes on the ensemble itself.
// Natural boundary conditions (the ensemble workload has no constraints).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ppf_gb300.h"
#include "handle.h"
#include "models.cuh"

#include <prismspf/gpu/cell_kernel_lanes.cuh>

namespace ppf {
namespace {

struct EnsInstance {
  int degree;
  int nc[2];
  int nn[2];
  long long N;
  long long off;      // offset of the instance's vectors in the packed arrays
  long long tab_off;  // offset (bytes, 16-aligned) of its CellTables in the packed tables
  double h[2];
  double m_well, kappa;
};

struct EnsLaunch {
  const EnsInstance* inst;
  const int* tile_inst;         // instance of each tile
  const long long* tile_cell0;  // first cell of each tile
  long long ntiles;
  const double* invm;
  const double* acc_in;
  double* acc_out;
  double* acc_zero;
  long long total_len;
  double dt;
  const unsigned char* tables;  // per-instance CellTables<2, degree, double>
  int fx;                       // integer derivatives (the tables enable them for Q1/Q2)
};

template <int degree, int CPB>
__device__ void ens_tile(const EnsLaunch& P, const EnsInstance& I, long long cell0, double* smem) {
  constexpr int n = degree + 1, nq = n * n;
  using Tab = pg::CellTables<2, degree, double>;
  Tab* tab = reinterpret_cast<Tab*>(smem);
  double* vals = smem + (sizeof(Tab) + 7) / 8;
  double* outs = vals + CPB * nq;
  long long* vals_fx = reinterpret_cast<long long*>(outs + 3 * CPB * nq);  // integer derivatives
  int* ex_in = reinterpret_cast<int*>(vals_fx + CPB * nq);                 // per-cell block exponent
  int* ex_out = ex_in + CPB;                                               // of the submitted terms
  const int t = threadIdx.x;
  // last read before the previous tile's closing barrier
  if (P.fx && t < CPB) {
    ex_in[t] = 0;
    ex_out[t] = 0;
  }
  // stage the instance's tables (built on the host for its mesh spacing)
  {
    const unsigned int* src = reinterpret_cast<const unsigned int*>(P.tables + I.tab_off);
    unsigned int* dst = reinterpret_cast<unsigned int*>(tab);
    for (int k = t; k < (int)(sizeof(Tab) / 4); k += blockDim.x) dst[k] = src[k];
  }
  const int lc = t / nq, q = t - lc * nq;
  const bool in_tile = lc < CPB;
  const long long cell = cell0 + lc;
  const long long ncells = (long long)I.nc[0] * I.nc[1];
  const bool active = in_tile && cell < ncells;
  const int qa = q % n, qb = q / n;
  long long node = 0;
  int cx = 0, cy = 0;
  if (active) {
    // instances hold fewer than 2^31 cells (int32 DoF indices): 32-bit division
    const unsigned int cl = (unsigned int)cell, n0 = (unsigned int)I.nc[0];
    cy = (int)(cl / n0);
    cx = (int)(cl - (unsigned int)cy * n0);
    node = (long long)(degree * cy + qb) * I.nn[0] + (degree * cx + qa);
    // gather: n = invM (.) acc of the previous step
    const double v = P.invm[I.off + node] * P.acc_in[I.off + node];
    vals[lc * nq + q] = v;
    if (P.fx) atomicMax(&ex_in[lc], pg::fx::exponent(v));
  }
  if (in_tile)
    for (int r = 0; r < 3; ++r) outs[r * CPB * nq + lc * nq + q] = 0.0;
  __syncthreads();
  if (P.fx) {
    // fixed-point copy of the nodal values for exact integer derivatives (fixed_point.cuh)
    if (active) {
      const int E = ex_in[lc];
      if (E != pg::fx::EXP_NONFINITE) vals_fx[lc * nq + q] = pg::fx::to_fixed(vals[lc * nq + q], E, pg::fx::TOP_VALUES);
    }
    __syncthreads();
  }
  pg::CellCtx<2, degree, double> ctx;
  ctx.tab = tab;
  ctx.vals = vals;
  ctx.outs = outs;
  ctx.stride = CPB * nq;
  ctx.lc = lc;
  ctx.q = q;
  ctx.cell[0] = cx;
  ctx.cell[1] = cy;
  ctx.cell[2] = 0;
  ctx.err = nullptr;
  ctx.submitted = 0;
  // integer integration of the value and gradient terms where the tables allow it (square cells):
  // the lane kernel's arithmetic (prismspf/gpu/cell_kernel_lanes.cuh) on this layout
  const bool fxi = P.fx && tab->fx_lanes;
  if (P.fx) {
    ctx.vals_fx = vals_fx;
    ctx.ex_in = ex_in;
    ctx.cpb = CPB;
    ctx.raw_values = fxi ? 1 : 0;
  }
  if (active) {
    AllenCahn<2, degree, double> pde{I.m_well, I.kappa};
    FieldContainer<2, degree, double> fc(ctx);
    pde.compute_rhs(fc, SimulationTimer(P.dt, 0.0), 1u);
  }
  __syncthreads();
  if (fxi) {
    namespace fx = pg::fx;
    constexpr int TOPT = LANE_TOP_TERMS;
    const int S = CPB * nq;
    const int p = lc * nq + q;
    if (active) {
      // block exponent of the cell's terms: the value term as h v, the two gradient terms
      const int ev = fx::exponent(outs[p]);
      const int eh = ev + tab->hk + (tab->hpow2 ? 0 : 1);
      int e = ev == 0 ? 0 : (ev == fx::EXP_NONFINITE || eh >= fx::EXP_NONFINITE ? fx::EXP_NONFINITE : max(eh, 0));
      e = max(e, fx::exponent(outs[S + p]));
      e = max(e, fx::exponent(outs[2 * S + p]));
      atomicMax(&ex_out[lc], e);
    }
    __syncthreads();
    long long* ox = reinterpret_cast<long long*>(outs);
    if (active) {
      const int E = ex_out[lc];
      const double v = outs[p];
      ox[p] = tab->hpow2 ? fx::to_fixed_fast<TOPT>(v, E - tab->hk) : fx::to_fixed_scaled<TOPT>(v, E, tab->hsig, tab->hk);
      ox[S + p] = fx::to_fixed_fast<TOPT>(outs[S + p], E);
      ox[2 * S + p] = fx::to_fixed_fast<TOPT>(outs[2 * S + p], E);
    }
    __syncthreads();
    if (active) {
      const int E = ex_out[lc];
      long long T = (long long)((unsigned long long)ox[p] << tab->vw_sh[q]);
      {
        const long long* g = ox + S + lc * nq + (q - qa);
        const long long L = lane_line_integral<n>(qa, g[0], g[1], n > 2 ? g[2] : 0ll);
        T += (long long)((unsigned long long)L << tab->wo_sh[0][q]);
      }
      {
        const long long* g = ox + 2 * S + lc * nq + (q - qb * n);
        const long long L = lane_line_integral<n>(qb, g[0], g[n], n > 2 ? g[2 * n] : 0ll);
        T += (long long)((unsigned long long)L << tab->wo_sh[1][q]);
      }
      const double rr = fx::to_double_fast(T, E - 1023 - TOPT + tab->ik[0], tab->isig[0], true);
      atomicAdd(P.acc_out + I.off + node, E == fx::EXP_NONFINITE ? fx::quiet_nan() : rr);
    }
    __syncthreads();
    return;
  }
  if (active) {
    double r = outs[lc * nq + q];
    {
      const double* g = outs + 1 * CPB * nq + lc * nq + (q - qa);
      const double* w = tab->jdt[0][q];
#pragma unroll
      for (int j = 0; j < n; ++j) r = fma(w[j], g[j], r);
    }
    {
      const double* g = outs + 2 * CPB * nq + lc * nq + (q - qb * n);
      const double* w = tab->jdt[1][q];
#pragma unroll
      for (int j = 0; j < n; ++j) r = fma(w[j], g[j * n], r);
    }
    atomicAdd(P.acc_out + I.off + node, r);
  }
  __syncthreads();
}

template <int CPB1, int CPB2, int THREADS>
__global__ void __launch_bounds__(THREADS) ensemble_step_kernel(const EnsLaunch P) {
  extern __shared__ __align__(16) double ens_smem[];
  // zero the third accumulator (read one step earlier, untouched by this launch)
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P.total_len;
       i += (long long)gridDim.x * blockDim.x)
    P.acc_zero[i] = 0.0;
  for (long long tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
    const EnsInstance I = P.inst[P.tile_inst[tile]];
    const long long cell0 = P.tile_cell0[tile];
    if (I.degree == 1) ens_tile<1, CPB1>(P, I, cell0, ens_smem);
    else ens_tile<2, CPB2>(P, I, cell0, ens_smem);
  }
}

template <int CPB1, int CPB2>
size_t ens_smem_bytes() {
  // tables, values, three output rows, the fixed-point values and the per-cell exponents
  const size_t t1 = (sizeof(pg::CellTables<2, 1, double>) + 7) / 8 * 8 + 8 * 5 * CPB1 * 4 + 8 * CPB1;
  const size_t t2 = (sizeof(pg::CellTables<2, 2, double>) + 7) / 8 * 8 + 8 * 5 * CPB2 * 9 + 8 * CPB2;
  return std::max(t1, t2) + 64;
}

// extraction of the field values: n = invM (.) acc
__global__ void ensemble_extract_kernel(double* out, const double* invm, const double* acc, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = invm[i] * acc[i];
}

// tile-shape candidates: cells per tile for Q1 and for Q2, threads per block
struct Shape {
  int cpb1, cpb2, threads;
};
constexpr Shape SHAPES[] = {{64, 28, 256}, {32, 14, 128}, {16, 7, 64}};
constexpr int NSHAPES = 3;

typedef void (*EnsKernel)(const EnsLaunch);
EnsKernel kernel_for(int s) {
  switch (s) {
    case 0: return ensemble_step_kernel<64, 28, 256>;
    case 1: return ensemble_step_kernel<32, 14, 128>;
    default: return ensemble_step_kernel<16, 7, 64>;
  }
}
size_t smem_for(int s) {
  switch (s) {
    case 0: return ens_smem_bytes<64, 28>();
    case 1: return ens_smem_bytes<32, 14>();
    default: return ens_smem_bytes<16, 7>();
  }
}

}  // namespace
}  // namespace ppf

struct ppf_ensemble_s {
  int n = 0;
  std::vector<ppf::EnsInstance> h_inst;
  ppf::EnsInstance* d_inst = nullptr;
  long long total = 0;
  double* invm = nullptr;
  double* acc[3] = {nullptr, nullptr, nullptr};
  double* scratch = nullptr;
  int* tile_inst = nullptr;
  long long* tile_cell0 = nullptr;
  long long ntiles = 0;
  int shape = 0;
  int grid_mult = 4;
  int sms = 0;
  double dt = 0.0;
  long long step = 0;  // accumulator rotation counter
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_shape = -1, graph_grid = -1;
  long long graph_phase = -1;
  std::string err;
  double gl_w[2][3];
  double gl_D[2][3][3];
  unsigned char* d_tables = nullptr;  // per-instance CellTables, 16-byte aligned
  int fx = 0;                         // the instance tables enable integer derivatives
};

namespace ppf {
namespace {

int efail(ppf_ensemble e, int code, const std::string& m) {
  if (e) e->err = m;
  return code;
}

#define ENS_CUDA(e, call)                                                                            \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return efail(e, PPF_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// tile list for the current shape
int build_tiles(ppf_ensemble e) {
  const Shape sh = SHAPES[e->shape];
  std::vector<int> ti;
  std::vector<long long> tc;
  for (int i = 0; i < e->n; ++i) {
    const EnsInstance& I = e->h_inst[i];
    const long long nc = (long long)I.nc[0] * I.nc[1];
    const int cpb = I.degree == 1 ? sh.cpb1 : sh.cpb2;
    for (long long c = 0; c < nc; c += cpb) {
      ti.push_back(i);
      tc.push_back(c);
    }
  }
  // interleave instances so consecutive tiles (and thus the blocks of one wave) mix
  // instances of both degrees
  std::vector<size_t> order(ti.size());
  for (size_t k = 0; k < order.size(); ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    const long long ra = tc[a] / (e->h_inst[ti[a]].degree == 1 ? sh.cpb1 : sh.cpb2);
    const long long rb = tc[b] / (e->h_inst[ti[b]].degree == 1 ? sh.cpb1 : sh.cpb2);
    return ra < rb;
  });
  std::vector<int> ti2(ti.size());
  std::vector<long long> tc2(tc.size());
  for (size_t k = 0; k < order.size(); ++k) {
    ti2[k] = ti[order[k]];
    tc2[k] = tc[order[k]];
  }
  if (e->graph) {  // the captured steps point at the previous tile list
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  cudaFree(e->tile_inst);
  cudaFree(e->tile_cell0);
  e->ntiles = (long long)ti2.size();
  ENS_CUDA(e, cudaMalloc(&e->tile_inst, sizeof(int) * e->ntiles));
  ENS_CUDA(e, cudaMalloc(&e->tile_cell0, sizeof(long long) * e->ntiles));
  ENS_CUDA(e, cudaMemcpy(e->tile_inst, ti2.data(), sizeof(int) * e->ntiles, cudaMemcpyHostToDevice));
  ENS_CUDA(e, cudaMemcpy(e->tile_cell0, tc2.data(), sizeof(long long) * e->ntiles, cudaMemcpyHostToDevice));
  return PPF_OK;
}

EnsLaunch make_launch(ppf_ensemble e, long long step) {
  EnsLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.inst = e->d_inst;
  L.tile_inst = e->tile_inst;
  L.tile_cell0 = e->tile_cell0;
  L.ntiles = e->ntiles;
  L.invm = e->invm;
  L.acc_in = e->acc[step % 3];
  L.acc_out = e->acc[(step + 1) % 3];
  L.acc_zero = e->acc[(step + 2) % 3];
  L.total_len = e->total;
  L.dt = e->dt;
  L.tables = e->d_tables;
  L.fx = e->fx;
  return L;
}

int launch_step(ppf_ensemble e, long long step, cudaStream_t s) {
  EnsKernel k = kernel_for(e->shape);
  const size_t smem = smem_for(e->shape);
  long long grid = (long long)e->sms * e->grid_mult;
  grid = std::max<long long>(1, std::min(grid, e->ntiles));
  k<<<(unsigned)grid, SHAPES[e->shape].threads, smem, s>>>(make_launch(e, step));
  return cudaGetLastError() == cudaSuccess ? PPF_OK : efail(e, PPF_ERR_CUDA, "ensemble step launch failed");
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" {

int ppf_ensemble_create(int n_instances, const ppf_mesh_desc* meshes, const double* m_well, const double* kappa,
                        double dt, ppf_ensemble* out) {
  if (!out || n_instances < 1 || !meshes || !m_well || !kappa) return PPF_ERR_ARG;
  *out = nullptr;
  auto* e = new ppf_ensemble_s();
  e->n = n_instances;
  e->dt = dt;
  for (int deg = 1; deg <= 2; ++deg) {
    GLRule g = gauss_lobatto(deg + 1);
    for (int i = 0; i <= deg; ++i) {
      e->gl_w[deg - 1][i] = g.w[i];
      for (int j = 0; j <= deg; ++j) e->gl_D[deg - 1][i][j] = g.D[i][j];
    }
  }
  long long off = 0;
  std::vector<double> invm;
  std::vector<unsigned char> tables;
  // the instance tables: block 1 of the Allen-Cahn application reads old n (value and gradient)
  // and submits n's value and gradient terms
  signed char slot_of[pg::MAX_FIELDS][pg::NAGE], slot_comp0[pg::MAX_SLOTS], out_of[pg::MAX_FIELDS],
      out_row0[pg::MAX_OUTS];
  std::memset(slot_of, -1, sizeof(slot_of));
  std::memset(slot_comp0, 0, sizeof(slot_comp0));
  std::memset(out_of, -1, sizeof(out_of));
  std::memset(out_row0, 0, sizeof(out_row0));
  slot_of[0][1] = 0;
  out_of[0] = 0;
  for (int i = 0; i < n_instances; ++i) {
    const ppf_mesh_desc& m = meshes[i];
    if (m.dim != 2 || m.degree < 1 || m.degree > 2 || m.periodic[0] || m.periodic[1]) {
      delete e;
      return PPF_ERR_UNSUPPORTED;
    }
    EnsInstance I{};
    I.degree = m.degree;
    for (int d = 0; d < 2; ++d) {
      I.nc[d] = m.subdivisions[d] << m.global_refinement;
      I.nn[d] = m.degree * I.nc[d] + 1;
      I.h[d] = m.size[d] / I.nc[d];
    }
    I.N = (long long)I.nn[0] * I.nn[1];
    I.off = off;
    {
      const double lo[3] = {0.0, 0.0, 0.0}, hh[3] = {I.h[0], I.h[1], 1.0};
      auto tb = build_cell_tables(2, I.degree, 0, lo, hh, slot_of, slot_comp0, out_of, out_row0, 1u);
      if (tb.empty()) {
        delete e;
        return PPF_ERR_UNSUPPORTED;
      }
      I.tab_off = (long long)tables.size();
      const int tfx = I.degree == 1 ? reinterpret_cast<const pg::CellTables<2, 1, double>*>(tb.data())->fx
                                    : reinterpret_cast<const pg::CellTables<2, 2, double>*>(tb.data())->fx;
      e->fx = (i == 0 ? 1 : e->fx) & (tfx != 0 ? 1 : 0);
      tables.insert(tables.end(), tb.begin(), tb.end());
      tables.resize((tables.size() + 15) / 16 * 16, 0);
    }
    I.m_well = m_well[i];
    I.kappa = kappa[i];
    off += I.N;
    e->h_inst.push_back(I);
    // lumped mass of the instance (natural boundaries)
    std::vector<double> m1[2];
    for (int d = 0; d < 2; ++d) {
      m1[d].assign(I.nn[d], 0.0);
      for (int c = 0; c < I.nc[d]; ++c)
        for (int a = 0; a <= I.degree; ++a) m1[d][I.degree * c + a] += e->gl_w[I.degree - 1][a] * I.h[d];
    }
    for (int J = 0; J < I.nn[1]; ++J)
      for (int K = 0; K < I.nn[0]; ++K) invm.push_back(1.0 / (m1[0][K] * m1[1][J]));
  }
  e->total = off;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev);
  auto bail = [&](int code) {
    ppf_ensemble_destroy(e);
    return code;
  };
  if (cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking) != cudaSuccess) return bail(PPF_ERR_CUDA);
  e->stream = e->own_stream;
  if (cudaMalloc(&e->d_inst, sizeof(EnsInstance) * n_instances) != cudaSuccess) return bail(PPF_ERR_CUDA);
  cudaMemcpy(e->d_inst, e->h_inst.data(), sizeof(EnsInstance) * n_instances, cudaMemcpyHostToDevice);
  if (cudaMalloc(&e->d_tables, tables.size()) != cudaSuccess) return bail(PPF_ERR_CUDA);
  cudaMemcpy(e->d_tables, tables.data(), tables.size(), cudaMemcpyHostToDevice);
  if (cudaMalloc(&e->invm, sizeof(double) * off) != cudaSuccess) return bail(PPF_ERR_CUDA);
  cudaMemcpy(e->invm, invm.data(), sizeof(double) * off, cudaMemcpyHostToDevice);
  for (int k = 0; k < 3; ++k) {
    if (cudaMalloc(&e->acc[k], sizeof(double) * off) != cudaSuccess) return bail(PPF_ERR_CUDA);
    cudaMemset(e->acc[k], 0, sizeof(double) * off);
  }
  if (cudaMalloc(&e->scratch, sizeof(double) * off) != cudaSuccess) return bail(PPF_ERR_CUDA);
  for (int s = 0; s < NSHAPES; ++s)
    cudaFuncSetAttribute(kernel_for(s), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(s));
  if (build_tiles(e)) return bail(PPF_ERR_CUDA);
  *out = e;
  return PPF_OK;
}

void ppf_ensemble_destroy(ppf_ensemble e) {
  if (!e) return;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  cudaFree(e->d_inst);
  cudaFree(e->d_tables);
  cudaFree(e->invm);
  for (int k = 0; k < 3; ++k) cudaFree(e->acc[k]);
  cudaFree(e->scratch);
  cudaFree(e->tile_inst);
  cudaFree(e->tile_cell0);
  if (e->own_stream) cudaStreamDestroy(e->own_stream);
  delete e;
}

const char* ppf_ensemble_last_error(ppf_ensemble e) { return e ? e->err.c_str() : "null ensemble"; }

long long ppf_ensemble_instance_length(ppf_ensemble e, int i) {
  if (!e || i < 0 || i >= e->n) return -1;
  return e->h_inst[i].N;
}

// upload instance i's field (lattice order): the accumulator holds mass (.) n
int ppf_ensemble_upload(ppf_ensemble e, int i, const double* host) {
  if (!e || !host || i < 0 || i >= e->n) return PPF_ERR_ARG;
  const EnsInstance& I = e->h_inst[i];
  std::vector<double> im(I.N), acc(I.N);
  ENS_CUDA(e, cudaMemcpy(im.data(), e->invm + I.off, sizeof(double) * I.N, cudaMemcpyDeviceToHost));
  for (long long k = 0; k < I.N; ++k) acc[k] = host[k] / im[k];
  ENS_CUDA(e, cudaMemcpy(e->acc[e->step % 3] + I.off, acc.data(), sizeof(double) * I.N, cudaMemcpyHostToDevice));
  return PPF_OK;
}

int ppf_ensemble_download(ppf_ensemble e, int i, double* host) {
  if (!e || !host || i < 0 || i >= e->n) return PPF_ERR_ARG;
  const EnsInstance& I = e->h_inst[i];
  ensemble_extract_kernel<<<grid_for(I.N), 256, 0, e->stream>>>(e->scratch + I.off, e->invm + I.off,
                                                                  e->acc[e->step % 3] + I.off, I.N);
  ENS_CUDA(e, cudaGetLastError());
  ENS_CUDA(e, cudaMemcpyAsync(host, e->scratch + I.off, sizeof(double) * I.N, cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  return PPF_OK;
}

// advance every instance by n_steps explicit steps: one launch per step; with use_graph the
// steps are replayed from a captured graph of three steps (one accumulator rotation)
int ppf_ensemble_run(ppf_ensemble e, int n_steps, int use_graph) {
  if (!e || n_steps < 0) return PPF_ERR_ARG;
  int done = 0;
  if (use_graph) {
    const long long phase = e->step % 3;
    if (!e->graph || e->graph_shape != e->shape || e->graph_grid != e->grid_mult || e->graph_phase != phase) {
      if (e->graph) cudaGraphExecDestroy(e->graph);
      e->graph = nullptr;
      cudaGraph_t g;
      ENS_CUDA(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < 3; ++k) launch_step(e, e->step + k, e->stream);
      ENS_CUDA(e, cudaStreamEndCapture(e->stream, &g));
      ENS_CUDA(e, cudaGraphInstantiate(&e->graph, g, 0));
      cudaGraphDestroy(g);
      e->graph_shape = e->shape;
      e->graph_grid = e->grid_mult;
      e->graph_phase = phase;
    }
    while (n_steps - done >= 3) {
      ENS_CUDA(e, cudaGraphLaunch(e->graph, e->stream));
      done += 3;
      e->step += 3;  // phase unchanged
    }
  }
  for (; done < n_steps; ++done) {
    int rc = launch_step(e, e->step, e->stream);
    if (rc) return rc;
    e->step++;
  }
  return PPF_OK;
}

// autotuner: times each tile shape and grid size on `steps` steps of this ensemble (on a copy
// of the state, which is restored) and keeps the fastest; returns its time per step in ms
int ppf_ensemble_autotune(ppf_ensemble e, int steps, double* best_ms, int* best_shape, int* best_grid) {
  if (!e || steps < 1) return PPF_ERR_ARG;
  // save the state
  std::vector<double> save(e->total);
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  ENS_CUDA(e, cudaMemcpy(save.data(), e->acc[e->step % 3], sizeof(double) * e->total, cudaMemcpyDeviceToHost));
  const long long step0 = e->step;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 1e300;
  int bs = e->shape, bg = e->grid_mult;
  const int grids[] = {1, 2, 4, 8};
  for (int s = 0; s < NSHAPES; ++s) {
    e->shape = s;
    if (build_tiles(e)) return PPF_ERR_CUDA;
    for (int gm : grids) {
      e->grid_mult = gm;
      launch_step(e, e->step, e->stream);  // warm-up
      e->step++;
      cudaEventRecord(a, e->stream);
      for (int k = 0; k < steps; ++k) {
        launch_step(e, e->step, e->stream);
        e->step++;
      }
      cudaEventRecord(b, e->stream);
      cudaEventSynchronize(b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      if (ms / steps < best) {
        best = ms / steps;
        bs = s;
        bg = gm;
      }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  e->shape = bs;
  e->grid_mult = bg;
  if (build_tiles(e)) return PPF_ERR_CUDA;
  // restore the state
  e->step = step0;
  for (int k = 0; k < 3; ++k) ENS_CUDA(e, cudaMemset(e->acc[k], 0, sizeof(double) * e->total));
  ENS_CUDA(e, cudaMemcpy(e->acc[e->step % 3], save.data(), sizeof(double) * e->total, cudaMemcpyHostToDevice));
  if (best_ms) *best_ms = best;
  if (best_shape) *best_shape = bs;
  if (best_grid) *best_grid = bg;
  return PPF_OK;
}

int ppf_ensemble_synchronize(ppf_ensemble e) {
  if (!e) return PPF_ERR_ARG;
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  return PPF_OK;
}

int ppf_ensemble_set_stream(ppf_ensemble e, void* stream) {
  if (!e) return PPF_ERR_ARG;
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  e->stream = stream ? static_cast<cudaStream_t>(stream) : e->own_stream;
  return PPF_OK;
}

}  // extern "C"
