// Linear solves of a single-field Linear block: CG preconditioned by nothing, by Chebyshev on
// the fine operator, or by a geometric-multigrid V-cycle (LinearSolver + MGContext,
// include/prismspf/solvers/linear_solver.h:47-553).
//
//   * operator: the LHS cell kernel (MODE_LHS) on each level, src read with the level's
//     homogeneous constraints, output zero on constrained rows, scaled by invM^1/2 unless the
//     tolerance type is AbsoluteResidual (MFOperator::compute_operator, mf_operator.cc:17-32);
//   * diagonal: unit probes (MODE_DIAG), same scaling, zero entries set to one, inverted
//     (MFOperator::compute_diagonal + eval_matrix_diagonal, mf_operator.cc:82-255);
//   * Chebyshev smoother of the first kind on [lambda_max/range, lambda_max] with
//     lambda_max = 1.2 x the largest eigenvalue of the Lanczos matrix of eig_cg_iterations
//     CG steps (Jacobi-preconditioned) on the pattern (i mod 11) minus its mean;
//   * transfers: the Gauss-Lobatto nodal interpolation from a level to the next finer one,
//     applied axis by axis (prolongation) and its transpose (restriction); images of
//     periodic nodes are condensed onto their masters and constrained rows zeroed;
//   * V-cycle: pre-smooth from zero (vmult), residual, restrict, recurse, prolongate-add,
//     post-smooth (step); the coarsest level applies the smoother (MGCoarseGridApplySmoother);
//   * mixed precision: all levels but the coarsest in FP32 (smoother, level operators,
//     transfers); the coarsest level, the outer CG and its residuals and inner products FP64;
//   * solve: LinearSolver::solve_impl (linear_solver.h:305-345): rhs = S b_rhs - S A g with
//     g the Dirichlet values (plain read), CG from the previous homogeneous solution,
//     x = x_hom + g, constraints distributed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <string>
#include <vector>

#include "handle.h"

namespace ppf {

// ------------------------------------------------------------------------------------------
// vector kernels
// ------------------------------------------------------------------------------------------
template <typename T>
__global__ void axpby_kernel(long long n, double a, const T* __restrict__ x, double b, T* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = T(a * double(x[i]) + b * double(y[i]));
}

template <typename Tin, typename Tout>
__global__ void convert_kernel(long long n, const Tin* __restrict__ x, Tout* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = Tout(x[i]);
}

template <typename T>
__global__ void mul_kernel(long long n, const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = a[i] * b[i];
}

// per-block partial sums of x.y in FP64 (deterministic two-stage reduction)
template <typename T>
__global__ void dot_partial_kernel(long long n, const T* __restrict__ x, const T* __restrict__ y, double* partial) {
  __shared__ double s[256];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += double(x[i]) * double(y[i]);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void dot_final_kernel(int nb, double* partial) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += partial[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[nb] = s[0];
}

// dst = scale (.) acc on free rows, zero on constrained rows (per node scale, component blocks)
template <typename T>
__global__ void level_finalize_kernel(T* __restrict__ dst, const T* __restrict__ acc, const T* __restrict__ scale,
                                      const int* __restrict__ cmap, long long N) {
  const long long base = blockIdx.y * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const long long gi = base + i;
    const bool free_row = !cmap || cmap[gi] == (int)gi;
    dst[gi] = free_row ? (scale ? acc[gi] * scale[i] : acc[gi]) : T(0);
  }
}

// inverse diagonal: d = scale (.) acc, zero entries -> 1, inverted
template <typename T>
__global__ void inv_diag_kernel(T* __restrict__ inv, const T* __restrict__ acc, const T* __restrict__ scale, long long N) {
  const long long base = blockIdx.y * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const long long gi = base + i;
    T d = scale ? acc[gi] * scale[i] : acc[gi];
    if (d == T(0)) d = T(1);
    inv[gi] = T(1) / d;
  }
}

// periodic images add into their master, then images and Dirichlet rows are zeroed
template <typename T>
__global__ void condense_add_kernel(long long len, T* v, const int* __restrict__ cmap) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const int m = cmap[i];
    if (m >= 0 && m != (int)i) atomicAdd(v + m, v[i]);
  }
}
template <typename T>
__global__ void zero_constrained_kernel(long long len, T* v, const int* __restrict__ cmap) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    if (cmap[i] != (int)i) v[i] = T(0);
}
// images take their master's value (AffineConstraints::distribute with homogeneous rows)
template <typename T>
__global__ void copy_masters_kernel(long long len, T* v, const int* __restrict__ cmap) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const int m = cmap[i];
    if (m != (int)i) v[i] = m >= 0 ? v[m] : T(0);
  }
}

// one 1-D sparse operator along `axis`: out(i) = sum_k val[k] in(i with axis index col[k])
template <typename T>
__global__ void axis_csr_kernel(const T* __restrict__ in, T* __restrict__ out, int o0, int o1, int o2, int axis,
                                int in_axis_len, const int* __restrict__ ptr, const int* __restrict__ col,
                                const T* __restrict__ val) {
  const long long total = (long long)o0 * o1 * o2;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(idx % o0);
    const int i1 = (int)((idx / o0) % o1);
    const int i2 = (int)(idx / ((long long)o0 * o1));
    const int row = axis == 0 ? i0 : (axis == 1 ? i1 : i2);
    const int d0 = axis == 0 ? in_axis_len : o0;
    const int d1 = axis == 1 ? in_axis_len : o1;
    T s = T(0);
    for (int k = ptr[row]; k < ptr[row + 1]; ++k) {
      const int c = col[k];
      const long long j = axis == 0 ? ((long long)i2 * d1 + i1) * d0 + c
                        : axis == 1 ? ((long long)i2 * d1 + c) * d0 + i0
                                    : ((long long)c * d1 + i1) * d0 + i0;
      s += val[k] * in[j];
    }
    out[idx] = s;
  }
}

// Chebyshev update: u = c1 u + c2 P (b - Ax); x += u
template <typename T>
__global__ void cheb_update_kernel(long long n, T* __restrict__ x, T* __restrict__ u, const T* __restrict__ b,
                                   const T* __restrict__ Ax, const T* __restrict__ pinv, double c1, double c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T r = Ax ? b[i] - Ax[i] : b[i];
    const T ui = T(c1) * u[i] + T(c2) * pinv[i] * r;
    u[i] = ui;
    x[i] += ui;
  }
}

// CG kernels (FP64)
__global__ void cg_update_xr_kernel(long long n, double alpha, const double* __restrict__ p,
                                    const double* __restrict__ q, double* __restrict__ x, double* __restrict__ r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    r[i] -= alpha * q[i];
  }
}

// ------------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------------
static size_t esize(int precision) { return precision ? sizeof(float) : sizeof(double); }

template <typename F>
static void by_precision(int precision, F&& f) {
  if (precision) f(float(0));
  else f(double(0));
}

static int dot(ppf_handle h, LinearState& L, int precision, long long n, const void* x, const void* y, double* out) {
  const unsigned nb = std::min<long long>(1024, (n + 255) / 256) > 0 ? (unsigned)std::min<long long>(1024, (n + 255) / 256) : 1;
  if (precision)
    dot_partial_kernel<float><<<nb, 256, 0, h->stream>>>(n, (const float*)x, (const float*)y, L.partial);
  else
    dot_partial_kernel<double><<<nb, 256, 0, h->stream>>>(n, (const double*)x, (const double*)y, L.partial);
  dot_final_kernel<<<1, 256, 0, h->stream>>>((int)nb, L.partial);
  h->all_launches += 2;
  PPF_CUDA(h, cudaMemcpyAsync(out, L.partial + nb, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  return PPF_OK;
}

static void axpby(ppf_handle h, int precision, long long n, double a, const void* x, double b, void* y) {
  if (precision) axpby_kernel<float><<<grid_for(n), 256, 0, h->stream>>>(n, a, (const float*)x, b, (float*)y);
  else axpby_kernel<double><<<grid_for(n), 256, 0, h->stream>>>(n, a, (const double*)x, b, (double*)y);
  h->all_launches++;
}

static void convert(ppf_handle h, int pin, int pout, long long n, const void* x, void* y) {
  if (pin == pout) {
    cudaMemcpyAsync(y, x, n * esize(pin), cudaMemcpyDeviceToDevice, h->stream);
    return;
  }
  if (pin == 0) convert_kernel<double, float><<<grid_for(n), 256, 0, h->stream>>>(n, (const double*)x, (float*)y);
  else convert_kernel<float, double><<<grid_for(n), 256, 0, h->stream>>>(n, (const float*)x, (double*)y);
  h->all_launches++;
}

// lumped mass on a lattice of nc cells per axis (periodic images condensed), inverted sqrt
// ------------------------------------------------------------------------------------------
// level set-up on the device (constraint map, inverse mass root, eigenvalue-estimate pattern)
// ------------------------------------------------------------------------------------------
struct LevelGeom {
  int nn[3];
  int periodic[3];
  int dim;
  long long N;
};

// pass 1: periodic images fold onto the lower face; free nodes on a Dirichlet face of their
// component (bit b of dmask[c]) become Dirichlet rows (-1)
__global__ void level_cmap_kernel(int* __restrict__ cm, LevelGeom g, int ncomp, unsigned dm0, unsigned dm1,
                                  unsigned dm2) {
  const long long len = ncomp * g.N;
  for (long long gi = blockIdx.x * (long long)blockDim.x + threadIdx.x; gi < len;
       gi += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(gi / g.N);
    const long long i = gi - c * g.N;
    long long I[3] = {i % g.nn[0], (i / g.nn[0]) % g.nn[1], i / ((long long)g.nn[0] * g.nn[1])};
    long long F[3] = {I[0], I[1], I[2]};
    for (int d = 0; d < g.dim; ++d)
      if (g.periodic[d] && F[d] == g.nn[d] - 1) F[d] = 0;
    const long long m = c * g.N + (F[2] * g.nn[1] + F[1]) * g.nn[0] + F[0];
    int v = (int)m;
    if (m == gi) {
      const unsigned dm = c == 0 ? dm0 : (c == 1 ? dm1 : dm2);
      for (int b = 0; b < 2 * g.dim; ++b)
        if ((dm >> b) & 1u) {
          const int d = b / 2;
          if ((b % 2 == 0 && I[d] == 0) || (b % 2 == 1 && I[d] == g.nn[d] - 1)) v = -1;
        }
    }
    cm[gi] = v;
  }
}

// pass 2: an image whose master is a Dirichlet row becomes a Dirichlet row
__global__ void level_cmap_close_kernel(int* __restrict__ cm, long long len) {
  for (long long gi = blockIdx.x * (long long)blockDim.x + threadIdx.x; gi < len;
       gi += (long long)gridDim.x * blockDim.x) {
    const int m = cm[gi];
    if (m >= 0 && m != (int)gi && cm[m] < 0) cm[gi] = -1;
  }
}

// invM^1/2 per node from the separable 1-D lumped masses m1 (axis d at m1 + off[d])
template <typename T>
__global__ void level_invm_sqrt_kernel(T* __restrict__ out, const double* __restrict__ m1, LevelGeom g, int off1,
                                       int off2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.N; i += (long long)gridDim.x * blockDim.x) {
    const long long I = i % g.nn[0], J = (i / g.nn[0]) % g.nn[1], K = i / ((long long)g.nn[0] * g.nn[1]);
    double m = m1[I];
    if (g.dim > 1) m *= m1[off1 + J];
    if (g.dim > 2) m *= m1[off2 + K];
    out[i] = m == 0.0 ? T(0) : T(sqrt(1.0 / m));
  }
}

// sum of (i mod 11) over free entries and their count (integers: exact in any order)
__global__ void pattern_sum_kernel(const int* __restrict__ cm, long long len, unsigned long long* sums) {
  unsigned long long s = 0, n = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    if (cm[i] == (int)i) {
      s += (unsigned long long)(i % 11);
      n += 1;
    }
  atomicAdd(sums, s);
  atomicAdd(sums + 1, n);
}

// the estimate's start vector: (i mod 11) - mean on free entries, zero on constrained ones
template <typename T>
__global__ void pattern_kernel(T* __restrict__ out, const int* __restrict__ cm, long long len, double mean) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    out[i] = cm[i] == (int)i ? T(double(i % 11) - mean) : T(0);
}

// 1-D prolongation from a coarse axis with ncc cells to the fine axis with 2 ncc cells
static void prolongation_1d(const GLRule& g, int k, int ncc, std::vector<int>& ptr, std::vector<int>& col,
                            std::vector<double>& val) {
  const int n = k + 1;
  const int nf = k * 2 * ncc + 1;
  ptr.assign(nf + 1, 0);
  col.clear();
  val.clear();
  for (int I = 0; I < nf; ++I) {
    const int cf = std::min(I / k, 2 * ncc - 1);
    const double xf = g.x[I - k * cf];
    const int cc = cf / 2;
    const double xc = ((cf % 2) + xf) * 0.5;
    for (int j = 0; j < n; ++j) {
      double L = 1.0;
      for (int m = 0; m < n; ++m)
        if (m != j) L *= (xc - g.x[m]) / (g.x[j] - g.x[m]);
      if (std::fabs(L) > 1e-14) {
        col.push_back(k * cc + j);
        val.push_back(L);
      }
    }
    ptr[I + 1] = (int)col.size();
  }
}

static void transpose_csr(int nrows, int ncols, const std::vector<int>& ptr, const std::vector<int>& col,
                          const std::vector<double>& val, std::vector<int>& tptr, std::vector<int>& tcol,
                          std::vector<double>& tval) {
  tptr.assign(ncols + 1, 0);
  for (int c : col) tptr[c + 1]++;
  for (int i = 0; i < ncols; ++i) tptr[i + 1] += tptr[i];
  tcol.assign(col.size(), 0);
  tval.assign(col.size(), 0.0);
  std::vector<int> pos(tptr.begin(), tptr.end() - 1);
  for (int r = 0; r < nrows; ++r)
    for (int q = ptr[r]; q < ptr[r + 1]; ++q) {
      const int p = pos[col[q]]++;
      tcol[p] = r;
      tval[p] = val[q];
    }
}

template <typename T>
static int upload_vec(ppf_handle h, void** dst, const std::vector<T>& v) {
  PPF_CUDA(h, cudaMalloc(dst, sizeof(T) * std::max<size_t>(1, v.size())));
  PPF_CUDA(h, cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return PPF_OK;
}

static int upload_real(ppf_handle h, void** dst, const std::vector<double>& v, int precision) {
  if (!precision) return upload_vec<double>(h, dst, v);
  std::vector<float> f(v.begin(), v.end());
  return upload_vec<float>(h, dst, f);
}

// ------------------------------------------------------------------------------------------
// level operators
// ------------------------------------------------------------------------------------------
// Contraction mode of the multigrid operators (levels and the outer FP64 operator):
// PPF_CONTRACTION_MODE if set, else the LHS plan's timed choice if a plain launch made one,
// else integer derivatives with FP64 integration.
static int multigrid_fx_mode(const BlockPlan& P, bool lanes_ok) {
  if (const int m = env_fx_mode(lanes_ok)) return m;
  return P.fx_mode > 0 && (P.fx_mode != 4 || lanes_ok) ? P.fx_mode : 1;
}

// Online choice of a contraction mode: the first 2 nm plain launches of an operator run modes
// 1 .. nm (nm = 3, or 4 where the lane kernel applies) twice under CUDA events (real work: the
// modes agree to rounding), then the fastest stays in `state`. begin returns the mode of this
// launch and the event slot (-1: not timed); end records the closing event and decides after
// the last timed launch.
static int online_mode_begin(ppf_handle h, int& state, int timed, cudaEvent_t* ev, int fallback, int* slot,
                             int nm) {
  *slot = -1;
  if (state > 0) return state;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &cs) != cudaSuccess || h->capturing || cs != cudaStreamCaptureStatusNone) {
    state = fallback;  // no timing (nor event waits) inside a graph capture
    return state;
  }
  *slot = timed;
  for (int i = 2 * timed; i < 2 * timed + 2; ++i)
    if (!ev[i] && cudaEventCreate(&ev[i]) != cudaSuccess) {
      *slot = -1;
      state = fallback;
      return state;
    }
  cudaEventRecord(ev[2 * timed], h->stream);
  return 1 + timed % nm;
}

static int online_mode_end(ppf_handle h, int& state, int& timed, cudaEvent_t* ev, int slot, int nm) {
  if (slot < 0) return PPF_OK;
  PPF_CUDA(h, cudaEventRecord(ev[2 * slot + 1], h->stream));
  if (++timed < 2 * nm) return PPF_OK;
  PPF_CUDA(h, cudaEventSynchronize(ev[4 * nm - 1]));
  float best[4] = {1e30f, 1e30f, 1e30f, 1e30f};
  for (int k = 0; k < 2 * nm; ++k) {
    float t = 0.f;
    PPF_CUDA(h, cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]));
    best[k % nm] = std::min(best[k % nm], t);
  }
  int b = 0;
  for (int k = 1; k < nm; ++k)
    if (best[k] < best[b]) b = k;
  state = 1 + b;
  for (int i = 0; i < 16; ++i) {
    if (ev[i]) cudaEventDestroy(ev[i]);
    ev[i] = nullptr;
  }
  return PPF_OK;
}

static int level_cell_launch(ppf_handle h, BlockState& B, MGLevel& lv, int mode, const void* src, bool plain_read) {
  const int f = B.desc.field_indices[0];
  FieldState& F = h->fields[f];
  CellLaunch L;
  std::memset(&L, 0, sizeof(L));
  for (int d = 0; d < 3; ++d) {
    L.nc[d] = lv.nc[d];
    L.nn[d] = lv.nn[d];
  }
  L.N = lv.N;
  L.ncells = lv.ncells;
  const BlockPlan& P = B.plan[1];
  L.nslots = P.nslots;
  for (int s = 0; s < P.nslots; ++s) {
    SlotDesc& sd = L.slots[s];
    sd.ncomp = h->fields[P.slot_field[s]].ncomp;
    if (P.slot_age[s] == 5) {
      sd.ptr = src;
      sd.is_src = 1;
      sd.out_index = 0;
      sd.constrained_read = plain_read ? 0 : (lv.constrained ? 1 : 0);
      sd.cmap = lv.cmap;
    } else {
      // other dependencies exist on the problem lattice only (FP64 single-level solves)
      sd.ptr = state_ptr(h, P.slot_field[s], P.slot_age[s]);
    }
  }
  L.nout = 1;
  L.outs[0].acc = lv.acc;
  L.outs[0].cmap = lv.constrained ? lv.cmap : nullptr;
  L.outs[0].ncomp = F.ncomp;
  L.nrows_in = P.nrows_in;
  L.nrows_out = P.nrows_out;
  L.tables = lv.tables;
  L.tables_host = lv.h_tables.data();
  L.timer = h->timer;
  L.block_id = (unsigned)B.desc.id;
  L.err = h->d_err;
  // integer contractions where the level's tables allow them (FP64 Q1/Q2); the mode is timed
  // online over the level's first plain LHS launches, so choosing costs no extra launches
  int slot = -1;
  const int nm = lv.fx_lanes ? 4 : 3;
  int m = multigrid_fx_mode(P, lv.fx_lanes);
  const bool fixed = env_fx_mode(lv.fx_lanes) != 0;
  if (P.fx && lv.precision == 0 && mode == MODE_LHS && !fixed)
    m = online_mode_begin(h, lv.fx_mode, lv.fx_timed, lv.fx_ev, 1, &slot, nm);
  set_fx_mode(L, m);
  // FP32 levels (mixed precision) run the FP32 lane kernel unless PPF_CONTRACTION_MODE fixes one
  // of the thread-block modes 1-3
  if (lv.precision == 1) {
    const int e = env_fx_mode(true);
    L.fx_lanes = e == 0 || e == 4;
  }
  const size_t smem = cell_smem(h->dim, h->k, lv.precision, P.nrows_in, P.nrows_out);
  const void* obj = lv.precision ? h->model_obj_f32.data() : h->model_obj.data();
  PPF_CUDA(h, cudaMemsetAsync(lv.acc, 0, lv.len * esize(lv.precision), h->stream));
  if (slot >= 0) PPF_CUDA(h, cudaEventRecord(lv.fx_ev[2 * slot], h->stream));  // after the memset
  const int rc = timed_cell_launch(h, lv.precision, mode, L, obj, smem);
  if (rc) return rc;
  return online_mode_end(h, lv.fx_mode, lv.fx_timed, lv.fx_ev, slot, nm);
}

static bool scaled(const LinearState& L) { return L.params.tolerance_type != 0; }

// dst = S A src on level lv (S = invM^1/2 or identity)
static int level_apply(ppf_handle h, BlockState& B, MGLevel& lv, const void* src, void* dst, bool plain_read = false) {
  int rc = level_cell_launch(h, B, lv, MODE_LHS, src, plain_read);
  if (rc) return rc;
  dim3 grid(grid_for(lv.N), h->fields[B.desc.field_indices[0]].ncomp);
  const int* cm = lv.constrained ? lv.cmap : nullptr;
  const bool sc = scaled(B.lin);
  if (lv.precision)
    level_finalize_kernel<float><<<grid, 256, 0, h->stream>>>((float*)dst, (const float*)lv.acc,
                                                              sc ? (const float*)lv.invm_sqrt : nullptr, cm, lv.N);
  else
    level_finalize_kernel<double><<<grid, 256, 0, h->stream>>>((double*)dst, (const double*)lv.acc,
                                                               sc ? (const double*)lv.invm_sqrt : nullptr, cm, lv.N);
  h->all_launches++;
  PPF_CUDA(h, cudaGetLastError());
  return PPF_OK;
}

static int level_diagonal(ppf_handle h, BlockState& B, MGLevel& lv) {
  int rc = level_cell_launch(h, B, lv, MODE_DIAG, lv.x, false);
  if (rc) return rc;
  dim3 grid(grid_for(lv.N), h->fields[B.desc.field_indices[0]].ncomp);
  const bool sc = scaled(B.lin);
  if (lv.precision)
    inv_diag_kernel<float><<<grid, 256, 0, h->stream>>>((float*)lv.inv_diag, (const float*)lv.acc,
                                                        sc ? (const float*)lv.invm_sqrt : nullptr, lv.N);
  else
    inv_diag_kernel<double><<<grid, 256, 0, h->stream>>>((double*)lv.inv_diag, (const double*)lv.acc,
                                                         sc ? (const double*)lv.invm_sqrt : nullptr, lv.N);
  h->all_launches++;
  PPF_CUDA(h, cudaGetLastError());
  return PPF_OK;
}

// largest eigenvalue of the symmetric tridiagonal (diag a, off-diagonal b) by bisection
static double tridiag_max_eig(const std::vector<double>& a, const std::vector<double>& b) {
  const int m = (int)a.size();
  if (m == 0) return 1.0;
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  auto count_below = [&](double x) {  // Sturm count of eigenvalues < x
    int cnt = 0;
    double q = a[0] - x;
    if (q < 0) cnt++;
    for (int i = 1; i < m; ++i) {
      const double qq = q == 0.0 ? 1e-300 : q;
      q = a[i] - x - b[i - 1] * b[i - 1] / qq;
      if (q < 0) cnt++;
    }
    return cnt;
  };
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (count_below(mid) >= m) hi = mid;
    else lo = mid;
    if (hi - lo <= 1e-14 * std::max(1.0, std::fabs(hi))) break;
  }
  return hi;
}

// Lanczos estimate of the largest eigenvalue of P A (P = inverse diagonal) on level lv:
// eig_cg_iterations CG steps on A x = pattern from x = 0 (uses lv.x, lv.b, lv.r, lv.w0, lv.w1)
template <typename T>
static int estimate_eigenvalues(ppf_handle h, BlockState& B, MGLevel& lv) {
  LinearState& L = B.lin;
  const int prec = lv.precision;
  {
    unsigned long long* d_sums = reinterpret_cast<unsigned long long*>(L.partial);
    PPF_CUDA(h, cudaMemsetAsync(d_sums, 0, 2 * sizeof(unsigned long long), h->stream));
    pattern_sum_kernel<<<grid_for(lv.len), 256, 0, h->stream>>>(lv.cmap, lv.len, d_sums);
    unsigned long long sums[2];
    PPF_CUDA(h, cudaMemcpyAsync(sums, d_sums, sizeof(sums), cudaMemcpyDeviceToHost, h->stream));
    PPF_CUDA(h, cudaStreamSynchronize(h->stream));
    const double mean = double(sums[0]) / double(std::max<unsigned long long>(1, sums[1]));
    pattern_kernel<T><<<grid_for(lv.len), 256, 0, h->stream>>>((T*)lv.b, lv.cmap, lv.len, mean);
    h->all_launches += 2;
    PPF_CUDA(h, cudaGetLastError());
  }
  T* x = (T*)lv.x;
  T* r = (T*)lv.r;
  T* z = (T*)lv.w0;
  T* p = (T*)lv.w1;
  PPF_CUDA(h, cudaMemsetAsync(x, 0, sizeof(T) * lv.len, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(r, lv.b, sizeof(T) * lv.len, cudaMemcpyDeviceToDevice, h->stream));
  const long long n = lv.len;
  mul_kernel<T><<<grid_for(n), 256, 0, h->stream>>>(n, (const T*)lv.inv_diag, r, z);
  PPF_CUDA(h, cudaMemcpyAsync(p, z, sizeof(T) * n, cudaMemcpyDeviceToDevice, h->stream));
  double rz;
  int rc = dot(h, L, prec, n, r, z, &rz);
  if (rc) return rc;
  double r0;
  rc = dot(h, L, prec, n, r, r, &r0);
  if (rc) return rc;
  std::vector<double> alphas, betas;
  for (int it = 0; it < L.params.eig_cg_iterations; ++it) {
    rc = level_apply(h, B, lv, p, lv.b);  // b reused as q = A p (pattern no longer needed)
    if (rc) return rc;
    double pq;
    rc = dot(h, L, prec, n, p, lv.b, &pq);
    if (rc) return rc;
    if (pq <= 0.0 || !std::isfinite(pq)) break;
    const double alpha = rz / pq;
    axpby(h, prec, n, alpha, p, 1.0, x);
    axpby(h, prec, n, -alpha, lv.b, 1.0, r);
    alphas.push_back(alpha);
    double rr;
    rc = dot(h, L, prec, n, r, r, &rr);
    if (rc) return rc;
    if (std::sqrt(rr) < 1e-10 * std::sqrt(r0)) break;
    mul_kernel<T><<<grid_for(n), 256, 0, h->stream>>>(n, (const T*)lv.inv_diag, r, z);
    double rz_new;
    rc = dot(h, L, prec, n, r, z, &rz_new);
    if (rc) return rc;
    const double beta = rz_new / rz;
    rz = rz_new;
    betas.push_back(beta);
    axpby(h, prec, n, 1.0, z, beta, p);
  }
  // Lanczos matrix of the CG coefficients
  const int m = (int)alphas.size();
  std::vector<double> a(m), b(m > 0 ? m - 1 : 0);
  for (int i = 0; i < m; ++i) {
    a[i] = 1.0 / alphas[i] + (i > 0 ? betas[i - 1] / alphas[i - 1] : 0.0);
    if (i + 1 < m) b[i] = std::sqrt(std::max(0.0, betas[i])) / alphas[i];
  }
  const double est = tridiag_max_eig(a, b);
  lv.lambda_max = 1.2 * est;
  lv.lambda_min = lv.lambda_max / L.params.smoothing_range;
  lv.eig_done = true;
  return PPF_OK;
}

// Chebyshev smoother on level lv: x <- x + p(P A)(P (b - A x)); zero_start: x := 0 first
template <typename T>
static int chebyshev(ppf_handle h, BlockState& B, MGLevel& lv, bool zero_start) {
  const double theta = 0.5 * (lv.lambda_max + lv.lambda_min);
  const double delta = 0.5 * (lv.lambda_max - lv.lambda_min);
  const double sigma = theta / delta;
  const long long n = lv.len;
  T* x = (T*)lv.x;
  T* u = (T*)lv.w0;
  T* Ax = (T*)lv.r;
  if (zero_start) PPF_CUDA(h, cudaMemsetAsync(x, 0, sizeof(T) * n, h->stream));
  PPF_CUDA(h, cudaMemsetAsync(u, 0, sizeof(T) * n, h->stream));
  double rho_prev = 1.0 / sigma;
  for (int k = 0; k < B.lin.params.smoother_degree; ++k) {
    const T* ax = nullptr;
    if (!(zero_start && k == 0)) {
      int rc = level_apply(h, B, lv, x, Ax);
      if (rc) return rc;
      ax = Ax;
    }
    double c1, c2;
    if (k == 0) {
      c1 = 0.0;
      c2 = 1.0 / theta;
    } else {
      const double rho = 1.0 / (2.0 * sigma - rho_prev);
      c1 = rho * rho_prev;
      c2 = 2.0 * rho / delta;
      rho_prev = rho;
    }
    cheb_update_kernel<T><<<grid_for(n), 256, 0, h->stream>>>(n, x, u, (const T*)lv.b, ax, (const T*)lv.inv_diag, c1, c2);
    h->all_launches++;
  }
  PPF_CUDA(h, cudaGetLastError());
  return PPF_OK;
}

static int smooth(ppf_handle h, BlockState& B, MGLevel& lv, bool zero_start) {
  if (lv.precision) return chebyshev<float>(h, B, lv, zero_start);
  return chebyshev<double>(h, B, lv, zero_start);
}

// separable transfer between level c (coarse) and c+1 (fine), in precision `prec`
template <typename T>
static void transfer(ppf_handle h, MGLevel& cl, MGLevel& fl, const T* in, T* out, bool prolongate, int ncomp) {
  const int dim = h->dim;
  for (int comp = 0; comp < ncomp; ++comp) {
    const T* src = in + comp * (prolongate ? cl.N : fl.N);
    T* dst = out + comp * (prolongate ? fl.N : cl.N);
    int cur[3] = {1, 1, 1};
    for (int d = 0; d < 3; ++d) cur[d] = prolongate ? cl.nn[d] : fl.nn[d];
    const T* a = src;
    for (int d = 0; d < dim; ++d) {
      int nxt[3] = {cur[0], cur[1], cur[2]};
      nxt[d] = prolongate ? fl.nn[d] : cl.nn[d];
      T* b = (d == dim - 1) ? dst : (T*)((d % 2 == 0) ? fl.t0 : fl.t1);
      const int* ptr = prolongate ? cl.p_ptr[d] : cl.r_ptr[d];
      const int* col = prolongate ? cl.p_col[d] : cl.r_col[d];
      const T* val = (const T*)(prolongate ? cl.p_val[d] : cl.r_val[d]);
      const long long total = (long long)nxt[0] * nxt[1] * nxt[2];
      axis_csr_kernel<T><<<grid_for(total), 256, 0, h->stream>>>(a, b, nxt[0], nxt[1], nxt[2], d, cur[d], ptr, col, val);
      h->all_launches++;
      a = b;
      cur[d] = nxt[d];
    }
  }
}

// V-cycle on level l: lv.b holds the defect, lv.x receives the correction
static int vcycle(ppf_handle h, BlockState& B, int l) {
  auto& lvs = B.lin.levels;
  MGLevel& lv = lvs[l];
  const int ncomp = h->fields[B.desc.field_indices[0]].ncomp;
  if (l == 0) return smooth(h, B, lv, true);  // coarse: the smoother as coarse solver
  int rc = smooth(h, B, lv, true);
  if (rc) return rc;
  // residual t = b - A x into lv.r
  rc = level_apply(h, B, lv, lv.x, lv.r);
  if (rc) return rc;
  axpby(h, lv.precision, lv.len, 1.0, lv.b, -1.0, lv.r);
  MGLevel& cl = lvs[l - 1];
  // restrict in the fine precision; the coarse level may hold another precision
  void* cb = (cl.precision == lv.precision) ? cl.b : cl.cvt;
  if (lv.precision) transfer<float>(h, cl, lv, (const float*)lv.r, (float*)cb, false, ncomp);
  else transfer<double>(h, cl, lv, (const double*)lv.r, (double*)cb, false, ncomp);
  if (cl.constrained) {
    if (lv.precision) {
      condense_add_kernel<float><<<grid_for(cl.len), 256, 0, h->stream>>>(cl.len, (float*)cb, cl.cmap);
      zero_constrained_kernel<float><<<grid_for(cl.len), 256, 0, h->stream>>>(cl.len, (float*)cb, cl.cmap);
    } else {
      condense_add_kernel<double><<<grid_for(cl.len), 256, 0, h->stream>>>(cl.len, (double*)cb, cl.cmap);
      zero_constrained_kernel<double><<<grid_for(cl.len), 256, 0, h->stream>>>(cl.len, (double*)cb, cl.cmap);
    }
    h->all_launches += 2;
  }
  if (cb != cl.b) convert(h, lv.precision, cl.precision, cl.len, cb, cl.b);
  rc = vcycle(h, B, l - 1);
  if (rc) return rc;
  // prolongate-add the coarse correction
  const void* cx = cl.x;
  if (cl.precision != lv.precision) {
    convert(h, cl.precision, lv.precision, cl.len, cl.x, cl.cvt);
    cx = cl.cvt;
  }
  if (lv.precision) transfer<float>(h, cl, lv, (const float*)cx, (float*)lv.r, true, ncomp);
  else transfer<double>(h, cl, lv, (const double*)cx, (double*)lv.r, true, ncomp);
  if (lv.constrained) {
    if (lv.precision) copy_masters_kernel<float><<<grid_for(lv.len), 256, 0, h->stream>>>(lv.len, (float*)lv.r, lv.cmap);
    else copy_masters_kernel<double><<<grid_for(lv.len), 256, 0, h->stream>>>(lv.len, (double*)lv.r, lv.cmap);
    h->all_launches++;
  }
  axpby(h, lv.precision, lv.len, 1.0, lv.r, 1.0, lv.x);
  return smooth(h, B, lv, false);
}

// ------------------------------------------------------------------------------------------
// set-up
// ------------------------------------------------------------------------------------------
static int alloc_real(ppf_handle h, void** p, long long n, int precision) {
  PPF_CUDA(h, cudaMalloc(p, std::max<long long>(1, n) * esize(precision)));
  PPF_CUDA(h, cudaMemset(*p, 0, std::max<long long>(1, n) * esize(precision)));
  return PPF_OK;
}

static int init_linear(ppf_handle h, int b) {
  BlockState& B = h->blocks[b];
  LinearState& L = B.lin;
  if (!L.params_set) {
    ppf_default_linear_params(&L.params);
    L.params_set = true;
  }
  if (B.desc.n_fields != 1) return fail(h, PPF_ERR_UNSUPPORTED, "linear blocks with more than one field");
  if (!B.plan[1].valid) return fail(h, PPF_ERR_ARG, "linear block has no LHS dependencies or no compiled LHS");
  for (int s = 0; s < B.plan[1].nslots; ++s)
    if (B.plan[1].slot_age[s] != 5 && L.params.preconditioner == 2)
      return fail(h, PPF_ERR_UNSUPPORTED, "GMG: the LHS may only depend on src in this build");
  const int f = B.desc.field_indices[0];
  FieldState& F = h->fields[f];
  const long long len = F.len;
  PPF_CUDA(h, cudaMalloc(&L.rhs, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.g, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.x_hom, sizeof(double) * len));
  PPF_CUDA(h, cudaMemset(L.x_hom, 0, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.r, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.p, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.q, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.z, sizeof(double) * len));
  PPF_CUDA(h, cudaMalloc(&L.partial, sizeof(double) * 1100));
  // levels: coarsest refinement R - depth + 1 .. R (depth 1 = the fine level only)
  const int R = h->mesh.global_refinement;
  int depth = L.params.preconditioner == 2 ? std::max(1, L.params.mg_depth) : 1;
  depth = std::min(depth, R + 1);
  L.levels.resize(depth);
  const GLRule g = gauss_lobatto(h->n);
  for (int l = 0; l < depth; ++l) {
    MGLevel& lv = L.levels[l];
    lv.refine = R - depth + 1 + l;
    lv.N = 1;
    lv.ncells = 1;
    for (int d = 0; d < 3; ++d) {
      if (d < h->dim) {
        lv.nc[d] = h->mesh.subdivisions[d] << lv.refine;
        lv.nn[d] = h->k * lv.nc[d] + 1;
        lv.h[d] = h->mesh.size[d] / lv.nc[d];
      } else {
        lv.nc[d] = lv.nn[d] = 1;
        lv.h[d] = 1.0;
      }
      lv.N *= lv.nn[d];
      lv.ncells *= lv.nc[d];
    }
    lv.len = F.ncomp * lv.N;
    const bool is_fine = l == depth - 1;
    lv.precision = (L.params.preconditioner == 2 && L.params.mixed_precision && l > 0) ? 1 : 0;
    // constraint map and invM^1/2 of the level, built on the device
    LevelGeom geom;
    geom.dim = h->dim;
    geom.N = lv.N;
    unsigned dmask[3] = {0u, 0u, 0u};
    bool any_constraint = false;
    for (int d = 0; d < 3; ++d) {
      geom.nn[d] = lv.nn[d];
      geom.periodic[d] = d < h->dim ? h->mesh.periodic[d] : 0;
      any_constraint |= geom.periodic[d] != 0;
    }
    for (int c = 0; c < F.ncomp; ++c)
      for (int bid = 0; bid < 2 * h->dim; ++bid)
        if (F.desc.dirichlet[c][bid]) {
          dmask[c] |= 1u << bid;
          any_constraint = true;
        }
    lv.constrained = any_constraint;
    PPF_CUDA(h, cudaMalloc(&lv.cmap, sizeof(int) * std::max<long long>(1, lv.len)));
    level_cmap_kernel<<<grid_for(lv.len), 256, 0, h->stream>>>(lv.cmap, geom, F.ncomp, dmask[0], dmask[1], dmask[2]);
    level_cmap_close_kernel<<<grid_for(lv.len), 256, 0, h->stream>>>(lv.cmap, lv.len);
    {
      std::vector<double> m1;
      int offs[3] = {0, 0, 0};
      for (int d = 0; d < h->dim; ++d) {
        offs[d] = (int)m1.size();
        std::vector<double> a(lv.nn[d], 0.0);
        for (int cc = 0; cc < lv.nc[d]; ++cc)
          for (int q = 0; q < h->n; ++q) a[h->k * cc + q] += g.w[q] * lv.h[d];
        if (h->mesh.periodic[d]) {
          a[0] += a[lv.nn[d] - 1];
          a[lv.nn[d] - 1] = 0.0;
        }
        m1.insert(m1.end(), a.begin(), a.end());
      }
      void* d_m1 = nullptr;
      int rc = upload_vec<double>(h, &d_m1, m1);
      if (rc) return rc;
      PPF_CUDA(h, cudaMalloc(&lv.invm_sqrt, esize(lv.precision) * std::max<long long>(1, lv.N)));
      if (lv.precision)
        level_invm_sqrt_kernel<float><<<grid_for(lv.N), 256, 0, h->stream>>>((float*)lv.invm_sqrt, (const double*)d_m1,
                                                                             geom, offs[1], offs[2]);
      else
        level_invm_sqrt_kernel<double><<<grid_for(lv.N), 256, 0, h->stream>>>((double*)lv.invm_sqrt,
                                                                              (const double*)d_m1, geom, offs[1], offs[2]);
      PPF_CUDA(h, cudaGetLastError());
      PPF_CUDA(h, cudaStreamSynchronize(h->stream));
      cudaFree(d_m1);
    }
    int rc = PPF_OK;
    // LHS tables of this level (the block's LHS dependency slots)
    signed char slot_of[pg::MAX_FIELDS][pg::NAGE];
    signed char slot_comp0[pg::MAX_SLOTS] = {};
    signed char out_of[pg::MAX_FIELDS];
    signed char out_row0[pg::MAX_OUTS] = {};
    std::memset(slot_of, -1, sizeof(slot_of));
    std::memset(out_of, -1, sizeof(out_of));
    int row = 0;
    for (int s = 0; s < B.plan[1].nslots; ++s) {
      slot_of[B.plan[1].slot_field[s]][B.plan[1].slot_age[s]] = (signed char)s;
      slot_comp0[s] = (signed char)row;
      row += h->fields[B.plan[1].slot_field[s]].ncomp;
    }
    out_of[f] = 0;
    double lo[3] = {h->mesh.lower[0], h->mesh.lower[1], h->mesh.lower[2]};
    auto tab = build_cell_tables(h->dim, h->k, lv.precision, lo, lv.h, slot_of, slot_comp0, out_of, out_row0,
                                 B.plan[1].fx_rows, B.plan[1].val_rows);
    PPF_CUDA(h, cudaMalloc(&lv.tables, tab.size()));
    PPF_CUDA(h, cudaMemcpy(lv.tables, tab.data(), tab.size(), cudaMemcpyHostToDevice));
    lv.fx_lanes = lv.precision == 0 && tables_lanes(tab, h->dim, h->k);
    lv.h_tables = std::move(tab);
    for (void** p : {&lv.inv_diag, &lv.acc, &lv.x, &lv.b, &lv.r, &lv.w0, &lv.w1}) {
      rc = alloc_real(h, p, lv.len, lv.precision);
      if (rc) return rc;
    }
    (void)is_fine;
  }
  // transfers between consecutive levels (stored on the coarse level; work buffers on the fine)
  for (int l = 0; l + 1 < depth; ++l) {
    MGLevel& cl = L.levels[l];
    MGLevel& fl = L.levels[l + 1];
    const int tp = fl.precision;  // transfers run in the fine level's precision
    for (int d = 0; d < h->dim; ++d) {
      std::vector<int> ptr, col, tptr, tcol;
      std::vector<double> val, tval;
      prolongation_1d(g, h->k, cl.nc[d], ptr, col, val);
      transpose_csr(fl.nn[d], cl.nn[d], ptr, col, val, tptr, tcol, tval);
      int rc = upload_vec<int>(h, (void**)&cl.p_ptr[d], ptr);
      if (!rc) rc = upload_vec<int>(h, (void**)&cl.p_col[d], col);
      if (!rc) rc = upload_real(h, &cl.p_val[d], val, tp);
      if (!rc) rc = upload_vec<int>(h, (void**)&cl.r_ptr[d], tptr);
      if (!rc) rc = upload_vec<int>(h, (void**)&cl.r_col[d], tcol);
      if (!rc) rc = upload_real(h, &cl.r_val[d], tval, tp);
      if (rc) return rc;
    }
    int rc = alloc_real(h, &fl.t0, fl.N, tp);
    if (!rc) rc = alloc_real(h, &fl.t1, fl.N, tp);
    if (rc) return rc;
    if (cl.precision != tp) {  // conversion buffer of coarse size in the transfer precision
      rc = alloc_real(h, &cl.cvt, cl.len, tp);
      if (rc) return rc;
    }
  }
  PPF_CUDA(h, cudaDeviceSynchronize());
  L.initialized = true;
  return PPF_OK;
}

// LinearSolver::normalization_value (linear_solver.h:414-427)
static double normalization(ppf_handle h, const LinearState& L, int n_fields = 1) {
  double v = 1.0;
  const int t = L.params.tolerance_type;
  if (t == 1 || t == 3) {
    double vol = 1.0;
    for (int d = 0; d < h->dim; ++d) vol *= h->mesh.size[d];
    v *= std::sqrt(vol);
  }
  if (t == 1 || t == 2) v *= std::sqrt((double)n_fields);
  return v;
}

// preconditioner application z = M^-1 r (FP64 fine vectors)
static int precondition(ppf_handle h, BlockState& B, const double* r, double* z) {
  LinearState& L = B.lin;
  const long long n = h->fields[B.desc.field_indices[0]].len;
  if (L.params.preconditioner == 0) {
    PPF_CUDA(h, cudaMemcpyAsync(z, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    return PPF_OK;
  }
  MGLevel& fine = L.levels.back();
  // the fine level's defect/solution vectors carry the V-cycle (or the Chebyshev smoother)
  convert(h, 0, fine.precision, n, r, fine.b);
  int rc = L.params.preconditioner == 1 ? smooth(h, B, fine, true) : vcycle(h, B, (int)L.levels.size() - 1);
  if (rc) return rc;
  convert(h, fine.precision, 0, n, fine.x, z);
  return PPF_OK;
}

// precondition() through a CUDA graph: the first application of a solve runs as plain
// launches (every kernel is configured then), the second is captured and every later one
// replays the graph: a V-cycle is a few hundred small launches on the coarse levels, whose
// launch overhead the graph removes. The graph holds the solve's simulation time and level
// state, so it is rebuilt for each solve.
static void drop_pc_graph(LinearState& L) {
  if (L.pc_graph) cudaGraphExecDestroy(L.pc_graph);
  L.pc_graph = nullptr;
  L.pc_calls = 0;
}

static int precondition_graphed(ppf_handle h, BlockState& B, const double* r, double* z) {
  LinearState& L = B.lin;
  if (L.params.preconditioner == 0 || h->timing || !h->use_graph || L.pc_nograph) return precondition(h, B, r, z);
  if (L.pc_graph && L.pc_in == r && L.pc_out == z) {
    PPF_CUDA(h, cudaGraphLaunch(L.pc_graph, h->stream));
    h->all_launches++;
    return PPF_OK;
  }
  if (L.pc_calls++ == 0) return precondition(h, B, r, z);
  drop_pc_graph(L);
  L.pc_calls = 2;
  if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    L.pc_nograph = true;
    return precondition(h, B, r, z);
  }
  int rc = precondition(h, B, r, z);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(h, PPF_ERR_CUDA, std::string("preconditioner capture: ") + cudaGetErrorString(e));
  const cudaError_t ie = cudaGraphInstantiate(&L.pc_graph, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) return fail(h, PPF_ERR_CUDA, std::string("preconditioner graph: ") + cudaGetErrorString(ie));
  L.pc_in = r;
  L.pc_out = z;
  PPF_CUDA(h, cudaGraphLaunch(L.pc_graph, h->stream));
  h->all_launches++;
  return PPF_OK;
}

int linear_solve(ppf_handle h, int b) {
  BlockState& B = h->blocks[b];
  LinearState& L = B.lin;
  L.last_init_ms = 0.0;
  if (h->amr) {
    // adaptive meshes: CG without a preconditioner on the current mesh's vectors, which are
    // re-made (warm start from zero) whenever the mesh changes
    if (!L.params_set) {
      ppf_default_linear_params(&L.params);
      L.params_set = true;
    }
    if (L.params.preconditioner != 0)
      return fail(h, PPF_ERR_UNSUPPORTED, "adaptive meshes: linear solves run without a preconditioner");
    if (B.desc.n_fields != 1) return fail(h, PPF_ERR_UNSUPPORTED, "linear blocks with more than one field");
    if (!B.plan[1].valid) return fail(h, PPF_ERR_ARG, "linear block has no LHS dependencies or no compiled LHS");
    if (L.mesh_version != h->mesh_version || !L.initialized) {
      const long long len = h->fields[B.desc.field_indices[0]].len;
      double** vecs[] = {&L.rhs, &L.g, &L.x_hom, &L.r, &L.p, &L.q, &L.z};
      for (double** v : vecs) {
        cudaFree(*v);
        *v = nullptr;
        PPF_CUDA(h, cudaMalloc(v, sizeof(double) * len));
      }
      PPF_CUDA(h, cudaMemsetAsync(L.x_hom, 0, sizeof(double) * len, h->stream));
      if (!L.partial) PPF_CUDA(h, cudaMalloc(&L.partial, sizeof(double) * 1100));
      L.mesh_version = h->mesh_version;
      L.initialized = true;
    }
  } else if (!L.initialized) {
    const auto t0 = std::chrono::steady_clock::now();
    int rc = init_linear(h, b);
    if (rc) return rc;
    L.last_init_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  const int f = B.desc.field_indices[0];
  FieldState& F = h->fields[f];
  const long long n = F.len;
  // FP64 outer operator on the problem lattice (the handle's FP64 LHS plan), also when the
  // fine multigrid level runs in FP32
  auto outer_apply = [&](const double* src, double* dst, bool plain) -> int {
    const double* srcs[PPF_MAX_FIELDS] = {src};
    PPF_CUDA(h, cudaMemsetAsync(F.acc, 0, sizeof(double) * n, h->stream));
    if (h->amr) {
      int rc = launch_cell(h, b, 1, srcs, plain);
      if (rc) return rc;
      dim3 grid(grid_for(h->N), F.ncomp);
      level_finalize_kernel<double><<<grid, 256, 0, h->stream>>>(dst, F.acc, scaled(L) ? h->d_invm_sqrt : nullptr,
                                                                 F.constrained ? F.cmap : nullptr, h->N);
      h->all_launches++;
      PPF_CUDA(h, cudaGetLastError());
      return PPF_OK;
    }
    CellLaunch Lc;
    std::memset(&Lc, 0, sizeof(Lc));
    for (int d = 0; d < 3; ++d) {
      Lc.nc[d] = h->nc[d];
      Lc.nn[d] = h->nn[d];
    }
    Lc.N = h->N;
    Lc.ncells = h->ncells;
    BlockPlan& P = B.plan[1];
    Lc.nslots = P.nslots;
    for (int s = 0; s < P.nslots; ++s) {
      SlotDesc& sd = Lc.slots[s];
      const int sf = P.slot_field[s];
      sd.ncomp = h->fields[sf].ncomp;
      if (P.slot_age[s] == 5) {
        sd.ptr = srcs[0];
        sd.constrained_read = plain ? 0 : (F.constrained ? 1 : 0);
        sd.cmap = F.cmap;
        sd.is_src = 1;
      } else {
        sd.ptr = state_ptr(h, sf, P.slot_age[s]);
      }
    }
    Lc.nout = 1;
    Lc.outs[0].acc = F.acc;
    Lc.outs[0].cmap = F.constrained ? F.cmap : nullptr;
    Lc.outs[0].ncomp = F.ncomp;
    Lc.nrows_in = P.nrows_in;
    Lc.nrows_out = P.nrows_out;
    Lc.tables = P.d_tables;
    Lc.tables_host = P.h_tables.data();
    Lc.timer = h->timer;
    Lc.block_id = (unsigned)B.desc.id;
    Lc.err = h->d_err;
    // the finest level is this operator on the same mesh: its timed mode if it has one; else
    // (an FP32 finest level) the plan's own mode, timed online over its first outer launches
    int slot = -1;
    const int nm = P.fx_lanes ? 4 : 3;
    {
      const int lm = L.levels.empty() ? -1 : L.levels.back().fx_mode;
      const bool fixed = env_fx_mode(P.fx_lanes) != 0;
      int m = multigrid_fx_mode(P, P.fx_lanes);
      if (!fixed && lm > 0 && (lm != 4 || P.fx_lanes)) m = lm;
      else if (!fixed && P.fx) m = online_mode_begin(h, P.fx_mode, P.fx_timed, P.fx_ev, 1, &slot, nm);
      set_fx_mode(Lc, m);
    }
    const size_t smem = cell_smem(h->dim, h->k, 0, P.nrows_in, P.nrows_out);
    int rc = timed_cell_launch(h, 0, MODE_LHS, Lc, h->model_obj.data(), smem);
    if (rc) return rc;
    rc = online_mode_end(h, P.fx_mode, P.fx_timed, P.fx_ev, slot, nm);
    if (rc) return rc;
    dim3 grid(grid_for(h->N), F.ncomp);
    level_finalize_kernel<double><<<grid, 256, 0, h->stream>>>(dst, F.acc, scaled(L) ? h->d_invm_sqrt : nullptr,
                                                               F.constrained ? F.cmap : nullptr, h->N);
    h->all_launches++;
    PPF_CUDA(h, cudaGetLastError());
    return PPF_OK;
  };
  // phase timers (host wall clock; each phase ends on a stream synchronisation)
  auto now = [] { return std::chrono::steady_clock::now(); };
  auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };
  drop_pc_graph(L);
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  const auto t_start = now();
  // diagonals of every level (recomputed for each solve, as the reference does)
  if (L.params.preconditioner != 0) {
    for (auto& lv : L.levels) {
      int rc = level_diagonal(h, B, lv);
      if (rc) return rc;
      if (!lv.eig_done) {
        rc = lv.precision ? estimate_eigenvalues<float>(h, B, lv) : estimate_eigenvalues<double>(h, B, lv);
        if (rc) return rc;
      }
    }
  }
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  const auto t_setup = now();
  // rhs = S * compute_rhs
  {
    PPF_CUDA(h, cudaMemsetAsync(F.acc, 0, sizeof(double) * n, h->stream));
    if (B.plan[0].valid && B.plan[0].nslots >= 0) {
      int rc = launch_cell(h, b, 0, nullptr);
      if (rc) return rc;
    }
    dim3 grid(grid_for(h->N), F.ncomp);
    level_finalize_kernel<double><<<grid, 256, 0, h->stream>>>(L.rhs, F.acc, scaled(L) ? h->d_invm_sqrt : nullptr,
                                                               F.constrained ? F.cmap : nullptr, h->N);
    h->all_launches++;
  }
  // inhomogeneous Dirichlet values g and rhs -= S A_plain g
  PPF_CUDA(h, cudaMemsetAsync(L.g, 0, sizeof(double) * n, h->stream));
  bool has_inhom = false;
  for (double v : F.h_dvals) has_inhom |= v != 0.0;
  if (has_inhom) {
    std::vector<double> gh(n, 0.0);
    for (long long i = 0; i < n; ++i)
      if (F.h_cmap[i] < 0) gh[i] = F.h_dvals[-1 - F.h_cmap[i]];
    if (h->amr) amr_fill_hanging(h, F.ncomp, gh.data());  // hanging nodes on Dirichlet faces
    PPF_CUDA(h, cudaMemcpyAsync(L.g, gh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    PPF_CUDA(h, cudaStreamSynchronize(h->stream));
    int rc = outer_apply(L.g, L.q, true);
    if (rc) return rc;
    axpby(h, 0, n, -1.0, L.q, 1.0, L.rhs);
  }
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  const auto t_rhs = now();
  // CG on S A x = rhs from the previous homogeneous solution (SolverCG)
  double* x = L.x_hom;
  const double tol = L.params.tolerance * normalization(h, L);
  int rc = outer_apply(x, L.q, false);
  if (rc) return rc;
  PPF_CUDA(h, cudaMemcpyAsync(L.r, L.rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  axpby(h, 0, n, -1.0, L.q, 1.0, L.r);
  double rr;
  rc = dot(h, L, 0, n, L.r, L.r, &rr);
  if (rc) return rc;
  double res = std::sqrt(rr);
  int it = 0;
  bool converged = res < tol;
  if (!converged) {
    rc = precondition_graphed(h, B, L.r, L.z);
    if (rc) return rc;
    PPF_CUDA(h, cudaMemcpyAsync(L.p, L.z, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    double rz;
    rc = dot(h, L, 0, n, L.r, L.z, &rz);
    if (rc) return rc;
    while (it < L.params.max_iterations) {
      rc = outer_apply(L.p, L.q, false);
      if (rc) return rc;
      double pq;
      rc = dot(h, L, 0, n, L.p, L.q, &pq);
      if (rc) return rc;
      const double alpha = rz / pq;
      cg_update_xr_kernel<<<grid_for(n), 256, 0, h->stream>>>(n, alpha, L.p, L.q, x, L.r);
      h->all_launches++;
      ++it;
      rc = dot(h, L, 0, n, L.r, L.r, &rr);
      if (rc) return rc;
      res = std::sqrt(rr);
      if (!std::isfinite(res)) return fail(h, PPF_ERR_NAN, "non-finite residual in the linear solve");
      if (res < tol) {
        converged = true;
        break;
      }
      rc = precondition_graphed(h, B, L.r, L.z);
      if (rc) return rc;
      double rz_new;
      rc = dot(h, L, 0, n, L.r, L.z, &rz_new);
      if (rc) return rc;
      const double beta = rz_new / rz;
      rz = rz_new;
      axpby(h, 0, n, 1.0, L.z, beta, L.p);
    }
  }
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  const auto t_end = now();
  L.last_setup_ms = ms(t_start, t_setup);
  L.last_rhs_ms = ms(t_setup, t_rhs);
  L.last_iterate_ms = ms(t_rhs, t_end);
  L.last_iterations = it;
  L.last_residual = res / normalization(h, L);
  double bb;
  rc = dot(h, L, 0, n, L.rhs, L.rhs, &bb);
  if (rc) return rc;
  L.last_rhs_norm = std::sqrt(bb);
  // solution = x_hom + g, then constraints
  PPF_CUDA(h, cudaMemcpyAsync(F.cur, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  axpby(h, 0, n, 1.0, L.g, 1.0, F.cur);
  rc = ppf_apply_constraints(h, f);
  if (rc) return rc;
  rc = check_err(h);
  if (rc) return rc;
  if (!converged) return fail(h, PPF_ERR_NOCONV, "linear solver did not converge before max iterations");
  return PPF_OK;
}

// ------------------------------------------------------------------------------------------
// Newton solves over all fields of a block (NewtonSolver::solve_impl, newton_solver.h:73-156,
// with LinearSolver::do_linear_solve, linear_solver.h:348-402). Block vectors concatenate the
// block's fields in block order on the device.
// ------------------------------------------------------------------------------------------
// dst = S op(src) on the block (which 0: compute_rhs, 1: compute_lhs with src read through
// the homogeneous constraints); constrained rows zero
static int block_op(ppf_handle h, int b, int which, const double* src, double* dst) {
  return ppf_apply_device(h, b, which, src, dst, scaled(h->blocks[b].lin) ? 2 : 0);
}

// Krylov solve of S A x = rhs from the initial guess in x (SolverCG or SolverBicgstab);
// preconditioner: identity, or the fine-level Chebyshev smoother for a single-field block
static int block_krylov(ppf_handle h, int b, const double* rhs, double* x, double tol, int* its, bool* conv) {
  BlockState& B = h->blocks[b];
  LinearState& L = B.lin;
  const long long n = L.block_len;
  double** v = L.kv;
  auto A = [&](const double* in, double* out) { return block_op(h, b, 1, in, out); };
  auto M = [&](const double* in, double* out) -> int {
    if (L.params.preconditioner == 0) {
      PPF_CUDA(h, cudaMemcpyAsync(out, in, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      return PPF_OK;
    }
    return precondition(h, B, in, out);
  };
  double* r = v[0];
  double* q = v[1];
  int rc = A(x, q);
  if (rc) return rc;
  PPF_CUDA(h, cudaMemcpyAsync(r, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  axpby(h, 0, n, -1.0, q, 1.0, r);
  double rr;
  rc = dot(h, L, 0, n, r, r, &rr);
  if (rc) return rc;
  double res = std::sqrt(rr);
  int it = 0;
  *conv = res < tol;
  if (!*conv && L.params.solver_type == 0) {
    double* z = v[2];
    double* p = v[3];
    if ((rc = M(r, z))) return rc;
    PPF_CUDA(h, cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    double rz;
    if ((rc = dot(h, L, 0, n, r, z, &rz))) return rc;
    while (it < L.params.max_iterations) {
      if ((rc = A(p, q))) return rc;
      double pq;
      if ((rc = dot(h, L, 0, n, p, q, &pq))) return rc;
      const double alpha = rz / pq;
      cg_update_xr_kernel<<<grid_for(n), 256, 0, h->stream>>>(n, alpha, p, q, x, r);
      h->all_launches++;
      ++it;
      if ((rc = dot(h, L, 0, n, r, r, &rr))) return rc;
      res = std::sqrt(rr);
      if (!std::isfinite(res)) return fail(h, PPF_ERR_NAN, "non-finite residual in the linear solve");
      if (res < tol) {
        *conv = true;
        break;
      }
      if ((rc = M(r, z))) return rc;
      double rz_new;
      if ((rc = dot(h, L, 0, n, r, z, &rz_new))) return rc;
      const double beta = rz_new / rz;
      rz = rz_new;
      axpby(h, 0, n, 1.0, z, beta, p);
    }
  } else if (!*conv) {
    // BiCGStab (van der Vorst), right-preconditioned, with the half-step convergence check
    double* rbar = v[2];
    double* p = v[3];
    double* vv = v[4];
    double* y = v[5];
    double* sv = v[6];
    double* t = v[7];
    double* zz = q;  // q is free from here on
    PPF_CUDA(h, cudaMemcpyAsync(rbar, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
    PPF_CUDA(h, cudaMemsetAsync(p, 0, sizeof(double) * n, h->stream));
    PPF_CUDA(h, cudaMemsetAsync(vv, 0, sizeof(double) * n, h->stream));
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int restarts = 0;
    // a breakdown (rho or omega zero, or |alpha| > 1e10) restarts from the current iterate with
    // the exact residual, as deal.II's SolverBicgstab does (at most 10 times)
    auto restart = [&]() -> int {
      if ((rc = A(x, q))) return rc;
      PPF_CUDA(h, cudaMemcpyAsync(r, rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      axpby(h, 0, n, -1.0, q, 1.0, r);
      PPF_CUDA(h, cudaMemcpyAsync(rbar, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      PPF_CUDA(h, cudaMemsetAsync(p, 0, sizeof(double) * n, h->stream));
      PPF_CUDA(h, cudaMemsetAsync(vv, 0, sizeof(double) * n, h->stream));
      rho = alpha = omega = 1.0;
      return dot(h, L, 0, n, r, r, &rr);
    };
    // a breakdown right at convergence: the exact residual of the restart meets the tolerance
    auto restarted_converged = [&]() -> bool {
      res = std::sqrt(rr);
      return res < tol;
    };
    while (it < L.params.max_iterations) {
      double rho_new;
      if ((rc = dot(h, L, 0, n, rbar, r, &rho_new))) return rc;
      if (rho_new == 0.0 || omega == 0.0) {  // breakdown
        if (++restarts > 10) break;
        if ((rc = restart())) return rc;
        if (restarted_converged()) { *conv = true; break; }
        continue;
      }
      const double beta = (rho_new / rho) * (alpha / omega);
      rho = rho_new;
      axpby(h, 0, n, -omega, vv, 1.0, p);  // p = p - omega v
      axpby(h, 0, n, 1.0, r, beta, p);     // p = r + beta p
      if ((rc = M(p, y))) return rc;
      if ((rc = A(y, vv))) return rc;
      double sigma;
      if ((rc = dot(h, L, 0, n, rbar, vv, &sigma))) return rc;
      if (sigma == 0.0 || !(std::fabs(rho / sigma) <= 1e10)) {  // breakdown
        if (++restarts > 10) break;
        if ((rc = restart())) return rc;
        if (restarted_converged()) { *conv = true; break; }
        continue;
      }
      alpha = rho / sigma;
      PPF_CUDA(h, cudaMemcpyAsync(sv, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      axpby(h, 0, n, -alpha, vv, 1.0, sv);  // s = r - alpha v
      ++it;
      double ss;
      if ((rc = dot(h, L, 0, n, sv, sv, &ss))) return rc;
      if (!std::isfinite(ss)) return fail(h, PPF_ERR_NAN, "non-finite residual in the linear solve");
      if (std::sqrt(ss) < tol) {
        axpby(h, 0, n, alpha, y, 1.0, x);
        res = std::sqrt(ss);
        *conv = true;
        break;
      }
      if ((rc = M(sv, zz))) return rc;
      if ((rc = A(zz, t))) return rc;
      double tt, ts;
      if ((rc = dot(h, L, 0, n, t, t, &tt))) return rc;
      if ((rc = dot(h, L, 0, n, t, sv, &ts))) return rc;
      omega = tt > 0.0 ? ts / tt : 0.0;
      axpby(h, 0, n, alpha, y, 1.0, x);
      axpby(h, 0, n, omega, zz, 1.0, x);
      PPF_CUDA(h, cudaMemcpyAsync(r, sv, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
      axpby(h, 0, n, -omega, t, 1.0, r);  // r = s - omega t
      if ((rc = dot(h, L, 0, n, r, r, &rr))) return rc;
      res = std::sqrt(rr);
      if (res < tol) {
        *conv = true;
        break;
      }
    }
  }
  *its = it;
  return PPF_OK;
}

int newton_solve(ppf_handle h, int b) {
  BlockState& B = h->blocks[b];
  LinearState& L = B.lin;
  if (!L.params_set) {
    ppf_default_linear_params(&L.params);
    L.params_set = true;
  }
  const int nbf = B.desc.n_fields;
  if (!B.plan[0].valid || !B.plan[1].valid)
    return fail(h, PPF_ERR_ARG, "Newton block needs compute_rhs and compute_lhs dependencies");
  if (L.params.preconditioner == 2)
    return fail(h, PPF_ERR_UNSUPPORTED, "Newton blocks: GMG levels would need the current solution on every level");
  if (h->amr && L.params.preconditioner != 0)
    return fail(h, PPF_ERR_UNSUPPORTED, "adaptive meshes: Newton blocks run without a preconditioner");
  if (L.params.preconditioner == 1 && nbf != 1)
    return fail(h, PPF_ERR_UNSUPPORTED, "Newton blocks: the Chebyshev preconditioner needs a single-field block");
  if (L.params.preconditioner == 1 && !L.initialized) {
    int rc = init_linear(h, b);
    if (rc) return rc;
  }
  long long off[PPF_MAX_FIELDS + 1] = {0};
  for (int i = 0; i < nbf; ++i) off[i + 1] = off[i] + h->fields[B.desc.field_indices[i]].len;
  const long long n = off[nbf];
  if (L.block_len != n || L.mesh_version != h->mesh_version) {
    L.mesh_version = h->mesh_version;
    cudaFree(L.newton_update);
    for (double*& p : L.kv) cudaFree(p);
    PPF_CUDA(h, cudaMalloc(&L.newton_update, sizeof(double) * n));
    PPF_CUDA(h, cudaMemset(L.newton_update, 0, sizeof(double) * n));
    for (double*& p : L.kv) PPF_CUDA(h, cudaMalloc(&p, sizeof(double) * n));
    cudaFree(L.rhs);  // a Newton block's rhs vector holds its block residual
    PPF_CUDA(h, cudaMalloc(&L.rhs, sizeof(double) * n));
    if (!L.partial) PPF_CUDA(h, cudaMalloc(&L.partial, sizeof(double) * 1100));
    L.block_len = n;
  }
  double* R = L.rhs;
  // start from the previous solution (old_1 where the field keeps one)
  for (int i = 0; i < nbf; ++i) {
    FieldState& F = h->fields[B.desc.field_indices[i]];
    if (F.n_old > 0)
      PPF_CUDA(h, cudaMemcpyAsync(F.cur, F.old[0], sizeof(double) * F.len, cudaMemcpyDeviceToDevice, h->stream));
  }
  const double norm = normalization(h, L, nbf);
  const double tol = L.newton_tolerance * norm;
  const double lin_tol = L.params.tolerance * norm;
  double l2 = -1.0;
  int iter = 0, lin_total = 0;
  while (iter < L.newton_max_iterations) {
    for (int i = 0; i < nbf; ++i) {
      int rc = ppf_apply_constraints(h, B.desc.field_indices[i]);
      if (rc) return rc;
    }
    int rc = block_op(h, b, 0, nullptr, R);
    if (rc) return rc;
    double rr;
    if ((rc = dot(h, L, 0, n, R, R, &rr))) return rc;
    l2 = std::sqrt(rr);
    if (!std::isfinite(l2)) return fail(h, PPF_ERR_NAN, "non-finite Newton residual");
    if (!(l2 > tol)) break;
    if (L.params.preconditioner == 1) {  // fine-level diagonal of the current Jacobian
      MGLevel& fine = L.levels.back();
      if ((rc = level_diagonal(h, B, fine))) return rc;
      fine.eig_done = false;
      if ((rc = estimate_eigenvalues<double>(h, B, fine))) return rc;
    }
    int its = 0;
    bool conv = false;
    if ((rc = block_krylov(h, b, R, L.newton_update, lin_tol, &its, &conv))) return rc;
    lin_total += its;
    for (int i = 0; i < nbf; ++i) {
      FieldState& F = h->fields[B.desc.field_indices[i]];
      axpby(h, 0, F.len, L.newton_step, L.newton_update + off[i], 1.0, F.cur);
    }
    ++iter;
  }
  L.last_newton_iterations = iter;
  L.last_newton_linear_iterations = lin_total;
  L.last_newton_residual = l2 / norm;
  int rc = check_err(h);
  if (rc) return rc;
  if (iter >= L.newton_max_iterations) return fail(h, PPF_ERR_NOCONV, "Newton solver did not converge");
  return PPF_OK;
}

void free_linear(LinearState& L) {
  drop_pc_graph(L);
  for (double* p : {L.rhs, L.g, L.x_hom, L.r, L.p, L.q, L.z, L.inv_diag, L.partial, L.newton_update}) cudaFree(p);
  for (double*& p : L.kv) {
    cudaFree(p);
    p = nullptr;
  }
  L.newton_update = nullptr;
  L.block_len = 0;
  for (auto& lv : L.levels) {
    for (auto& ev : lv.fx_ev)
      if (ev) cudaEventDestroy(ev);
    cudaFree(lv.cmap);
    for (void* p : {lv.invm_sqrt, lv.inv_diag, lv.tables, lv.acc, lv.x, lv.b, lv.r, lv.w0, lv.w1, lv.t0, lv.t1, lv.cvt})
      cudaFree(p);
    for (int d = 0; d < 3; ++d) {
      cudaFree(lv.p_ptr[d]);
      cudaFree(lv.p_col[d]);
      cudaFree(lv.p_val[d]);
      cudaFree(lv.r_ptr[d]);
      cudaFree(lv.r_col[d]);
      cudaFree(lv.r_val[d]);
    }
  }
  L.levels.clear();
  L.initialized = false;
}

}  // namespace ppf

using namespace ppf;

extern "C" {

int ppf_default_linear_params(ppf_linear_params* p) {
  if (!p) return PPF_ERR_ARG;
  p->tolerance_type = 0;
  p->tolerance = 1e-10;
  p->max_iterations = 100;
  p->preconditioner = 0;
  p->mg_depth = 1;
  p->smoother_degree = 5;
  p->smoothing_range = 15.0;
  p->eig_cg_iterations = 10;
  p->mixed_precision = 0;
  p->solver_type = 0;
  return PPF_OK;
}

int ppf_set_linear_params(ppf_handle h, int b, const ppf_linear_params* p) {
  if (!h || !p || b < 0 || b >= (int)h->blocks.size()) return PPF_ERR_ARG;
  if (p->preconditioner < 0 || p->preconditioner > 2 || p->smoother_degree < 1 || p->mg_depth < 1 ||
      p->max_iterations < 1 || p->eig_cg_iterations < 1 || p->smoothing_range <= 1.0 || p->solver_type < 0 ||
      p->solver_type > 1)
    return fail(h, PPF_ERR_ARG, "invalid linear solver parameters");
  LinearState& L = h->blocks[b].lin;
  if (L.initialized) return fail(h, PPF_ERR_ARG, "linear parameters are fixed after the first solve");
  if (p->mixed_precision && h->model_obj_f32.empty())
    return fail(h, PPF_ERR_UNSUPPORTED, "mixed precision needs an FP32 instance of the operator");
  L.params = *p;
  L.params_set = true;
  return PPF_OK;
}

int ppf_linear_stats(ppf_handle h, int b, double* init_ms, double* setup_ms, double* rhs_ms, double* iterate_ms) {
  if (!h || b < 0 || b >= (int)h->blocks.size()) return PPF_ERR_ARG;
  const LinearState& L = h->blocks[b].lin;
  if (init_ms) *init_ms = L.last_init_ms;
  if (setup_ms) *setup_ms = L.last_setup_ms;
  if (rhs_ms) *rhs_ms = L.last_rhs_ms;
  if (iterate_ms) *iterate_ms = L.last_iterate_ms;
  return PPF_OK;
}

int ppf_set_newton_params(ppf_handle h, int b, int max_iterations, double tolerance, double step_length) {
  if (!h || b < 0 || b >= (int)h->blocks.size() || max_iterations < 1 || !(tolerance >= 0.0) || !(step_length > 0.0))
    return PPF_ERR_ARG;
  LinearState& L = h->blocks[b].lin;
  L.newton_max_iterations = max_iterations;
  L.newton_tolerance = tolerance;
  L.newton_step = step_length;
  return PPF_OK;
}

int ppf_newton_solve(ppf_handle h, int b, int* newton_iterations, int* linear_iterations, double* residual) {
  if (!h || b < 0 || b >= (int)h->blocks.size()) return PPF_ERR_ARG;
  if (h->blocks[b].desc.solve_type != PPF_NEWTON) return fail(h, PPF_ERR_ARG, "block is not Newton");
  const int rc = newton_solve(h, b);
  const LinearState& L = h->blocks[b].lin;
  if (newton_iterations) *newton_iterations = L.last_newton_iterations;
  if (linear_iterations) *linear_iterations = L.last_newton_linear_iterations;
  if (residual) *residual = L.last_newton_residual;
  return rc;
}

int ppf_linear_solve(ppf_handle h, int b, int* iterations, double* residual) {
  if (!h || b < 0 || b >= (int)h->blocks.size()) return PPF_ERR_ARG;
  if (h->blocks[b].desc.solve_type != PPF_LINEAR) return fail(h, PPF_ERR_ARG, "block is not Linear");
  const int rc = linear_solve(h, b);
  if (iterations) *iterations = h->blocks[b].lin.last_iterations;
  if (residual) *residual = h->blocks[b].lin.last_residual;
  return rc;
}

int ppf_lhs_diagonal(ppf_handle h, int b, double* out) {
  if (!h || !out || b < 0 || b >= (int)h->blocks.size()) return PPF_ERR_ARG;
  BlockState& B = h->blocks[b];
  if (!B.lin.initialized) {
    int rc = init_linear(h, b);
    if (rc) return rc;
  }
  MGLevel& fine = B.lin.levels.back();
  if (fine.precision) return fail(h, PPF_ERR_ARG, "diagonal export needs an FP64 fine level");
  int rc = level_diagonal(h, B, fine);
  if (rc) return rc;
  std::vector<double> inv(fine.len);
  PPF_CUDA(h, cudaMemcpyAsync(inv.data(), fine.inv_diag, sizeof(double) * fine.len, cudaMemcpyDeviceToHost, h->stream));
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  for (long long i = 0; i < fine.len; ++i) out[i] = 1.0 / inv[i];
  return check_err(h);
}

}  // extern "C"
