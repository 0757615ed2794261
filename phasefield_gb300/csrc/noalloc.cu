// Allocation-free explicit Allen-Cahn step.
//
// Who this is for: callers that cannot allocate GPU memory when they need a step, e.g. code
// that runs inside a host framework owning every device allocation through its own pool,
// or inside a fixed-memory real-time loop where cudaMalloc/cudaFree (which can synchronise
// the device and fragment a pre-sized pool) are not allowed. They hand over the input and
// output vectors they already own; this entry point needs no handle and calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// The step is the explicit solve of the Allen-Cahn application's block 1 (the same cell
// kernel and operator set as the handle path): accumulate the cell integrals, then scale by
// the inverse lumped mass. The accumulator, the per-call cell tables and the error word live
// in one file-scope __device__ array (g_noalloc_scratch) of fixed size, so the largest mesh
// is NOALLOC_MAX_NODES lattice nodes; larger meshes are rejected with PPF_ERR_UNSUPPORTED.
// Every GPU that loads this library holds that array (8 MiB + 32 KiB) until the process
// exits.
//
// Sharing: all calls on a device share the one array and it keeps the last call's contents;
// each call clears the accumulator and the error word before use. Two calls whose GPU work
// overlaps (different streams, or different host threads) race on the array, so callers
// serialise them, e.g. by issuing them on one stream.
//
// Set-up: the first call on a device, with that device current, looks up the device address
// of the array with cudaGetSymbolAddress and the device's SM count, and caches both per
// device. Make that first call before any stream capture begins.
//
// Status: the finalize kernel sets a non-finite flag in the array's error word; the step
// itself returns before its GPU work ends and so cannot report it.
// ppf_allen_cahn_step_noalloc_status waits for a stream and reads that word (a copy into a
// host int of the caller's stack, no allocation).
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/ppf_gb300.h"
#include "models.cuh"
#include "runtime.h"

namespace ppf {
namespace {

constexpr long long NOALLOC_MAX_NODES = 1LL << 20;  // 1,048,576 lattice nodes (8 MiB of FP64)
constexpr size_t NOALLOC_TABLE_BYTES = 32768;  // CellTables of any dim/degree (Q4 3-D: about 19 KB)
constexpr size_t NOALLOC_ACC_BYTES = (size_t)NOALLOC_MAX_NODES * sizeof(double);
constexpr size_t NOALLOC_BYTES = NOALLOC_ACC_BYTES + NOALLOC_TABLE_BYTES + 256;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr size_t NOALLOC_ERR_OFFSET = NOALLOC_ACC_BYTES + NOALLOC_TABLE_BYTES;

// device address of g_noalloc_scratch and the SM count, per device (host-side cache)
static unsigned char* g_scratch_addr[NOALLOC_MAX_DEVICES] = {};
static int g_sm_count[NOALLOC_MAX_DEVICES] = {};

// the cell tables travel as a kernel argument (kernel parameters of up to 32 KB are
// available from CUDA 12.1 on), so the call stages them without a host-to-device copy
template <size_t B>
struct alignas(16) TableBlob {
  unsigned char b[B];
};

template <size_t B>
__global__ void noalloc_stage_tables_kernel(const __grid_constant__ TableBlob<B> blob, unsigned char* dst,
                                            int* err) {
  for (int i = threadIdx.x; i < (int)B; i += blockDim.x) dst[i] = blob.b[i];
  if (threadIdx.x == 0) *err = 0;
}

int noalloc_fail(int code, const char* msg) {
  std::fprintf(stderr, "ppf_allen_cahn_step_noalloc: %s\n", msg);
  return code;
}

// Gauss-Lobatto nodes and weights on [0,1] in closed form for 2..5 points.
void gl_closed_form(int n, double* x, double* w) {
  const double s5 = 1.0 / std::sqrt(5.0), s37 = std::sqrt(3.0 / 7.0);
  switch (n) {
    case 2: x[0] = 0; x[1] = 1; w[0] = w[1] = 0.5; break;
    case 3: x[0] = 0; x[1] = 0.5; x[2] = 1; w[0] = w[2] = 1.0 / 6; w[1] = 2.0 / 3; break;
    case 4:
      x[0] = 0; x[1] = 0.5 * (1 - s5); x[2] = 0.5 * (1 + s5); x[3] = 1;
      w[0] = w[3] = 1.0 / 12; w[1] = w[2] = 5.0 / 12;
      break;
    default:
      x[0] = 0; x[1] = 0.5 * (1 - s37); x[2] = 0.5; x[3] = 0.5 * (1 + s37); x[4] = 1;
      w[0] = w[4] = 1.0 / 20; w[1] = w[3] = 49.0 / 180; w[2] = 16.0 / 45;
      break;
  }
}

// Builds the cell tables of block 1 and launches the kernel that writes them (and clears the
// error word) into the scratch array; returns false when that launch fails.
template <int dim, int degree>
bool stage_tables(const ppf_mesh_desc& m, const double* h, unsigned char* d_tables, int* d_err, cudaStream_t s) {
  using Tab = pg::CellTables<dim, degree>;
  static_assert(sizeof(Tab) <= NOALLOC_TABLE_BYTES, "cell tables exceed the scratch table region");
  static_assert(sizeof(Tab) <= 32000, "cell tables exceed the kernel-parameter limit");
  constexpr int n = degree + 1, nq = Tab::nq;
  TableBlob<sizeof(Tab)> blob;
  Tab& t = *reinterpret_cast<Tab*>(blob.b);
  std::memset(&t, 0, sizeof(Tab));
  double x[5], w[5], D[5][5], bw[5];
  gl_closed_form(n, x, w);
  for (int j = 0; j < n; ++j) {
    double p = 1.0;
    for (int k = 0; k < n; ++k)
      if (k != j) p *= x[j] - x[k];
    bw[j] = 1.0 / p;
  }
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j)
      if (j != i) {
        D[i][j] = bw[j] / (bw[i] * (x[i] - x[j]));
        diag -= D[i][j];
      }
    D[i][i] = diag;
  }
  double detJ = 1.0;
  for (int d = 0; d < dim; ++d) detJ *= h[d];
  for (int d = 0; d < dim; ++d)
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        t.Dh[d][i][j] = D[i][j] / h[d];
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += D[i][k] * D[k][j];
        t.D2h[d][i][j] = s / (h[d] * h[d]);
      }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) t.Dt[i][j] = D[j][i];
  for (int q = 0; q < nq; ++q) {
    double wq = detJ;
    int r = q;
    for (int d = 0; d < dim; ++d) {
      wq *= w[r % n];
      r /= n;
    }
    t.jxw[q] = wq;
  }
  for (int d = 0; d < dim; ++d) {
    const int sd = d == 0 ? 1 : (d == 1 ? n : n * n);
    for (int q = 0; q < nq; ++q) {
      const int id = (q / sd) % n;
      for (int j = 0; j < n; ++j) t.jdt[d][q][j] = D[j][id] * (t.jxw[q + (j - id) * sd] / h[d]);
    }
  }
  for (int d = 0; d < 3; ++d) {
    t.lo[d] = d < dim ? m.lower[d] : 0.0;
    t.h[d] = d < dim ? h[d] : 1.0;
  }
  for (int i = 0; i < n; ++i) t.gl_x[i] = x[i];
  t.vol = detJ;
  // dependency of block 1: old_1(n) values and gradients (slot 0); output: field 0
  std::memset(t.slot_of, -1, sizeof(t.slot_of));
  std::memset(t.out_of, -1, sizeof(t.out_of));
  t.slot_of[0][1] = 0;
  t.slot_comp0[0] = 0;
  t.out_of[0] = 0;
  t.out_row0[0] = 0;
  noalloc_stage_tables_kernel<sizeof(Tab)><<<1, 256, 0, s>>>(blob, d_tables, d_err);
  return cudaGetLastError() == cudaSuccess;
}

bool stage_tables_dispatch(int dim, int degree, const ppf_mesh_desc& m, const double* h, unsigned char* d_tables,
                           int* d_err, cudaStream_t s) {
  switch (dim * 10 + degree) {
    case 21: return stage_tables<2, 1>(m, h, d_tables, d_err, s);
    case 22: return stage_tables<2, 2>(m, h, d_tables, d_err, s);
    case 23: return stage_tables<2, 3>(m, h, d_tables, d_err, s);
    case 24: return stage_tables<2, 4>(m, h, d_tables, d_err, s);
    case 31: return stage_tables<3, 1>(m, h, d_tables, d_err, s);
    case 32: return stage_tables<3, 2>(m, h, d_tables, d_err, s);
    case 33: return stage_tables<3, 3>(m, h, d_tables, d_err, s);
    case 34: return stage_tables<3, 4>(m, h, d_tables, d_err, s);
    default: return false;
  }
}

struct LumpedMass1D {
  double w[5];
  int k;
  int nc[3];
  double h[3];
};

// u_new = acc / m, with the lumped mass m of a natural-boundary uniform mesh evaluated from
// the lattice indices: a product over directions of h_d times the GL weight of the node's
// position in its cell, doubled where two cells share the node.
__global__ void noalloc_finalize_kernel(double* __restrict__ u, const double* __restrict__ acc, const int nn0,
                                        const int nn1, const long long N, const LumpedMass1D m, const int dim,
                                        int* err) {
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    long long idx[3] = {i % nn0, (i / nn0) % nn1, i / ((long long)nn0 * nn1)};
    double mass = 1.0;
    for (int d = 0; d < dim; ++d) {
      const long long I = idx[d];
      const int a = (int)(I % m.k);
      double w1;
      if (a != 0) w1 = m.w[a];
      else if (I == 0 || I == (long long)m.k * m.nc[d]) w1 = m.w[0];
      else w1 = 2.0 * m.w[0];
      mass *= w1 * m.h[d];
    }
    const double v = acc[i] / mass;
    bad |= !isfinite(v);
    u[i] = v;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(err, int(pg::ERR_NONFINITE));
}

}  // namespace
}  // namespace ppf

using namespace ppf;

extern "C" int ppf_allen_cahn_step_noalloc(const ppf_mesh_desc* mesh, double m_well, double kappa, double dt,
                                           const double* d_n_old, double* d_n_new, void* stream) {
  if (!mesh || !d_n_old || !d_n_new) return noalloc_fail(PPF_ERR_ARG, "null argument");
  const int dim = mesh->dim, degree = mesh->degree;
  if (dim < 2 || dim > 3 || degree < 1 || degree > 4 || mesh->global_refinement < 0 ||
      mesh->global_refinement > 30)
    return noalloc_fail(PPF_ERR_ARG, "mesh: dim must be 2 or 3, degree 1..4, global refinement 0..30");
  for (int d = 0; d < dim; ++d) {
    if (mesh->periodic[d])
      return noalloc_fail(PPF_ERR_UNSUPPORTED, "allocation-free step: natural boundary conditions only");
    if (mesh->subdivisions[d] < 1 || mesh->size[d] <= 0) return noalloc_fail(PPF_ERR_ARG, "mesh: bad size");
  }
  int nc[3] = {1, 1, 1}, nn[3] = {1, 1, 1};
  double h[3] = {1, 1, 1};
  long long N = 1, ncells = 1;
  for (int d = 0; d < dim; ++d) {
    // counts in 64 bits: a large refinement must not wrap to a small mesh that passes the limit
    const long long cells = (long long)mesh->subdivisions[d] << mesh->global_refinement;
    if (cells > NOALLOC_MAX_NODES)
      return noalloc_fail(PPF_ERR_UNSUPPORTED,
                          "allocation-free step: mesh exceeds the 1048576-node limit of the static scratch array");
    nc[d] = (int)cells;
    nn[d] = degree * nc[d] + 1;
    h[d] = mesh->size[d] / nc[d];
    N *= nn[d];
    ncells *= nc[d];
    if (N > NOALLOC_MAX_NODES) break;
  }
  if (N > NOALLOC_MAX_NODES)
    return noalloc_fail(PPF_ERR_UNSUPPORTED,
                        "allocation-free step: mesh exceeds the 1048576-node limit of the static scratch array");
  const ModelOps* model = find_model("allen_cahn");
  if (!model) return noalloc_fail(PPF_ERR_UNSUPPORTED, "allen_cahn operator set not compiled in");

  // one-time set-up per device: device address of the static scratch array
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return noalloc_fail(PPF_ERR_CUDA, "no usable current CUDA device");
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return noalloc_fail(PPF_ERR_CUDA, "cudaGetSymbolAddress failed for the scratch array");
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
      return noalloc_fail(PPF_ERR_CUDA, "cudaDeviceGetAttribute failed for the SM count");
    g_sm_count[dev] = sms;
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  unsigned char* base = g_scratch_addr[dev];
  double* acc = reinterpret_cast<double*>(base);
  unsigned char* d_tables = base + NOALLOC_ACC_BYTES;
  int* d_err = reinterpret_cast<int*>(base + NOALLOC_ERR_OFFSET);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  AllenCahn<2, 1, double> pde{m_well, kappa};  // same layout for every dim/degree
  // tables and the cleared error word, then the cleared accumulator
  if (!stage_tables_dispatch(dim, degree, *mesh, h, d_tables, d_err, s))
    return noalloc_fail(PPF_ERR_CUDA, "staging the cell tables failed");
  if (cudaMemsetAsync(acc, 0, sizeof(double) * N, s) != cudaSuccess)
    return noalloc_fail(PPF_ERR_CUDA, "clearing the accumulator failed");

  CellLaunch L;
  std::memset(&L, 0, sizeof(L));
  for (int d = 0; d < 3; ++d) {
    L.nc[d] = nc[d];
    L.nn[d] = nn[d];
  }
  L.N = N;
  L.ncells = ncells;
  L.nslots = 1;
  L.slots[0].ptr = d_n_old;
  L.slots[0].ncomp = 1;
  L.nout = 1;
  L.outs[0].acc = acc;
  L.outs[0].ncomp = 1;
  L.nrows_in = 1;
  L.nrows_out = 1 + dim;
  L.tables = d_tables;
  L.timer = prismspf::SimulationTimer(dt, 0.0);
  L.block_id = 1;
  L.err = d_err;
  const size_t smem = cell_smem(dim, degree, 0, L.nrows_in, L.nrows_out);
  if (model->launch(dim, degree, MODE_RHS, 0, L, &pde, smem, s) != cudaSuccess)
    return noalloc_fail(PPF_ERR_CUDA, "cell kernel launch failed");

  LumpedMass1D lm{};
  double x[5];
  gl_closed_form(degree + 1, x, lm.w);
  lm.k = degree;
  for (int d = 0; d < 3; ++d) {
    lm.nc[d] = nc[d];
    lm.h[d] = h[d];
  }
  long long grid = (N + 255) / 256;
  if (grid > (long long)g_sm_count[dev] * 16) grid = (long long)g_sm_count[dev] * 16;
  noalloc_finalize_kernel<<<(unsigned)grid, 256, 0, s>>>(d_n_new, acc, nn[0], nn[1], N, lm, dim, d_err);
  if (cudaGetLastError() != cudaSuccess) return noalloc_fail(PPF_ERR_CUDA, "finalize kernel launch failed");
  return PPF_OK;
}

extern "C" int ppf_allen_cahn_step_noalloc_status(void* stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return noalloc_fail(PPF_ERR_CUDA, "no usable current CUDA device");
  if (!g_scratch_addr[dev]) return PPF_OK;  // no step has run on this device
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int flags = 0;
  if (cudaStreamSynchronize(s) != cudaSuccess ||
      cudaMemcpyFromSymbol(&flags, g_noalloc_scratch, sizeof(int), NOALLOC_ERR_OFFSET, cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return noalloc_fail(PPF_ERR_CUDA, "reading the error word failed");
  return (flags & pg::ERR_NONFINITE) ? PPF_ERR_NAN : PPF_OK;
}
