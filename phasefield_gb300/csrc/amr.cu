// Adaptive meshes on the GPU: the RefinementManager path (src/core/refinement_manager.cc:42-439)
// of a handle. The host keeps the forest (amr_mesh.cu) and rebuilds numbering, constraints and
// the transfer plan when the mesh changes; the device does the per-step work (cell kernel on the
// cell list, finalize with hanging-node distribution) and the per-remesh work (criteria on every
// cell, transfer of every stored age, constraint distribution).
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <prismspf/gpu/amr_cell_kernel.cuh>

#include "amr_mesh.h"
#include "handle.h"

namespace ppf {

constexpr int AMR_MAX_LEVELS = 20;

struct AmrCriterion {
  int field, flags;
  double vlo, vhi, glo;
};

struct AmrState {
  AmrMesh mesh;
  int min_level = 0, max_level = 0, period = 0, global_level = 0;
  std::vector<AmrCriterion> crit;
  int nlev = 0;                      // max_level - min_level + 1 level tables per plan
  std::vector<void*> d_tables;       // per block: rhs, lhs (nlev consecutive CellTables)
  int* d_cell_dofs = nullptr;
  int4* d_cell_info = nullptr;
  int* d_h_dof = nullptr;
  int* d_h_ptr = nullptr;
  int* d_h_idx = nullptr;
  double* d_h_w = nullptr;
  int nrows = 0;
  signed char* d_flags = nullptr;
  std::vector<ppf_dirichlet_fn> dfn;  // per field
  std::vector<void*> duser;
  // wall-clock phases of the last remeshing pass (ms): criteria, smoothing, new mesh
  // (refine, numbering, hanging lines, transfer plan), transfer (device vectors), set-up of the
  // new mesh (mesh arrays, invM, constraints, distribution)
  double phase_ms[5] = {0, 0, 0, 0, 0};
};

namespace {

// value of a free or Dirichlet row after the explicit update
__device__ __forceinline__ double amr_final_value(const double* __restrict__ acc, const double* __restrict__ invm,
                                                  const int* __restrict__ cmap, const double* __restrict__ dvals,
                                                  long long gi, long long i) {
  const int cm = cmap ? cmap[gi] : (int)gi;
  return cm == (int)gi ? invm[i] * acc[gi] : dvals[-1 - cm];
}

// The explicit update u = invM (.) acc followed by distribute(): free rows scale their
// accumulator, Dirichlet rows take their values, hanging rows the interpolant of their masters'
// final values (computed here from the masters' accumulators, so one launch does all rows; the
// reference's invM is 0 on hanging rows and distribute() sets them)
__global__ void amr_finalize_kernel(double* __restrict__ u, const double* __restrict__ acc,
                                    const double* __restrict__ invm, const int* __restrict__ cmap,
                                    const double* __restrict__ dvals, const int* __restrict__ h_ptr,
                                    const int* __restrict__ h_idx, const double* __restrict__ h_w, long long N,
                                    int* err) {
  const long long base = blockIdx.y * N;
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const long long gi = base + i;
    const int cm = cmap ? cmap[gi] : (int)gi;
    double v;
    if (cm >= AMR_HANG_BASE) {
      const int r = cm - AMR_HANG_BASE;
      v = 0.0;
      for (int e = h_ptr[r]; e < h_ptr[r + 1]; ++e) {
        const long long m = h_idx[e];
        v += h_w[e] * amr_final_value(acc, invm, cmap, dvals, base + m, m);
      }
    } else {
      v = cm == (int)gi ? invm[i] * acc[gi] : dvals[-1 - cm];
    }
    bad |= !isfinite(v);
    u[gi] = v;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(err, int(pg::ERR_NONFINITE));
}

// Dirichlet rows take their values (AffineConstraints::distribute, inhomogeneous part)
__global__ void amr_dirichlet_kernel(double* __restrict__ u, const int* __restrict__ cmap,
                                     const double* __restrict__ dvals, long long len) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const int cm = cmap[i];
    if (cm < 0) u[i] = dvals[-1 - cm];
  }
}

// hanging rows take the interpolant of their masters (free or Dirichlet, already final)
__global__ void amr_hanging_kernel(double* __restrict__ u, const int* __restrict__ h_dof, const int* __restrict__ h_ptr,
                                   const int* __restrict__ h_idx, const double* __restrict__ h_w, int nrows,
                                   long long N) {
  const long long base = blockIdx.y * N;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int e = h_ptr[r]; e < h_ptr[r + 1]; ++e) s += h_w[e] * u[base + h_idx[e]];
    u[base + h_dof[r]] = s;
  }
}

// new[c N + p] = sum_e w[e] old[c No + idx[e]] for the rows of the transfer plan
__global__ void amr_transfer_kernel(const int* __restrict__ ptr, const int* __restrict__ idx,
                                    const double* __restrict__ w, const double* __restrict__ old,
                                    double* __restrict__ nw, long long N, long long No) {
  const int c = blockIdx.y;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int e = ptr[p]; e < ptr[p + 1]; ++e) s += w[e] * old[c * No + idx[e]];
    nw[c * N + p] = s;
  }
}

struct MarkArgs {
  const double* u[PPF_MAX_FIELDS];
  int ncomp[PPF_MAX_FIELDS];
  int flags[PPF_MAX_FIELDS];
  double vlo[PPF_MAX_FIELDS], vhi[PPF_MAX_FIELDS], glo[PPF_MAX_FIELDS];
  int ncrit;
  double D[pg::MAX_N][pg::MAX_N];
  double h[AMR_MAX_LEVELS][3];  // cell size per level (from min_level)
  int dim, n, nq, min_level, max_level;
  long long N, ncells;
};

// RefinementManager::mark_cells_for_refinement_and_coarsening (refinement_manager.cc:161-363):
// one thread per cell evaluates every criterion at the cell's quadrature points (the GL nodes)
__global__ void amr_mark_kernel(const __grid_constant__ MarkArgs A, const int* __restrict__ cell_dofs,
                                const int4* __restrict__ info, signed char* __restrict__ flags) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < A.ncells;
       c += (long long)gridDim.x * blockDim.x) {
    const int4 in = info[c];
    const int lev = in.x + A.min_level;
    const int n = A.n, nq = A.nq;
    bool refine = false;
    for (int k = 0; k < A.ncrit && !refine; ++k) {
      const int ncomp = A.ncomp[k];
      for (int l = 0; l < nq && !refine; ++l) {
        if (A.flags[k] & PPF_REFINE_VALUE) {
          double v;
          if (ncomp == 1) {
            v = A.u[k][cell_dofs[c * nq + l]];
          } else {
            double s2 = 0.0;
            for (int cc = 0; cc < ncomp; ++cc) {
              const double x = A.u[k][cc * A.N + cell_dofs[c * nq + l]];
              s2 += x * x;
            }
            v = sqrt(s2);
          }
          if (v > A.vlo[k] && v < A.vhi[k]) refine = true;
        }
        if (!refine && (A.flags[k] & PPF_REFINE_GRADIENT)) {
          const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
          const int stride[3] = {1, n, n * n};
          double mag2 = 0.0;
          for (int cc = 0; cc < ncomp; ++cc) {
            double g2 = 0.0;
            for (int d = 0; d < A.dim; ++d) {
              const int base = l - idx[d] * stride[d];
              double acc = 0.0;
              for (int j = 0; j < n; ++j) acc += A.D[idx[d]][j] * A.u[k][cc * A.N + cell_dofs[c * nq + base + j * stride[d]]];
              const double g = acc / A.h[in.x][d];
              g2 += g * g;
            }
            if (ncomp == 1) {
              mag2 = g2;
            } else {
              const double gm = sqrt(g2);
              mag2 += gm * gm;
            }
          }
          const double mag = sqrt(mag2);
          if (ncomp == 1 ? mag > A.glo[k] : (mag > A.vlo[k] && mag < A.vhi[k])) refine = true;
        }
      }
    }
    flags[c] = refine ? (lev < A.max_level ? 1 : 0) : (lev > A.min_level ? -1 : 0);
  }
}

template <class T>
int upload_vec(ppf_handle h, T*& dst, const std::vector<T>& src) {
  cudaFree(dst);
  dst = nullptr;
  const size_t n = src.empty() ? 1 : src.size();
  PPF_CUDA(h, cudaMalloc(&dst, sizeof(T) * n));
  if (!src.empty()) {
    // on the handle's (non-blocking) stream, waited for: the host vector may go away next
    PPF_CUDA(h, cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, h->stream));
    PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return PPF_OK;
}

int upload_mesh(ppf_handle h) {
  AmrState& A = *h->amr;
  const AmrMesh& m = A.mesh;
  int rc = upload_vec(h, A.d_cell_dofs, m.cell_dofs);
  if (rc) return rc;
  std::vector<int4> info(m.cells.size());
  for (size_t c = 0; c < m.cells.size(); ++c)
    info[c] = make_int4(m.cells[c].lev - A.min_level, m.cells[c].x[0], m.cells[c].x[1], m.cells[c].x[2]);
  if ((rc = upload_vec(h, A.d_cell_info, info))) return rc;
  if ((rc = upload_vec(h, A.d_h_dof, m.h_dof))) return rc;
  if ((rc = upload_vec(h, A.d_h_ptr, m.h_ptr))) return rc;
  if ((rc = upload_vec(h, A.d_h_idx, m.h_idx))) return rc;
  if ((rc = upload_vec(h, A.d_h_w, m.h_w))) return rc;
  A.nrows = (int)m.h_dof.size();
  cudaFree(A.d_flags);
  A.d_flags = nullptr;
  PPF_CUDA(h, cudaMalloc(&A.d_flags, std::max<size_t>(1, m.cells.size())));
  h->N = m.N;
  h->ncells = m.ncells();
  return PPF_OK;
}

double level_h(const ppf_handle h, int d, int lev) {
  // the uniform mesh's expression size / (subdivisions 2^level), so level tables of the
  // initial level are identical to the uniform handle's
  return h->mesh.size[d] / (int)((long long)h->mesh.subdivisions[d] << lev);
}

// constraint map and Dirichlet values of field f on the current mesh
int build_constraints(ppf_handle h, int f) {
  AmrState& A = *h->amr;
  const AmrMesh& m = A.mesh;
  FieldState& F = h->fields[f];
  const long long N = m.N;
  F.h_cmap.assign(F.len, 0);
  F.h_dvals.clear();
  F.h_drow.clear();
  bool any = false;
  for (int c = 0; c < F.ncomp; ++c)
    for (long long p = 0; p < N; ++p) {
      const long long gi = c * N + p;
      F.h_cmap[gi] = m.hang_row[p] >= 0 ? AMR_HANG_BASE + m.hang_row[p] : (int)gi;
      any |= m.hang_row[p] >= 0;
    }
  // interpolate_boundary_values: boundary ids ascending, DoFs not yet constrained
  const double t = h->timer.get_time();
  for (int c = 0; c < F.ncomp; ++c)
    for (int b = 0; b < 2 * h->dim; ++b) {
      if (!F.desc.dirichlet[c][b]) continue;
      const int d = b / 2;
      if (m.periodic[d]) continue;
      const long long at = (b % 2 == 0) ? 0 : m.E[d];
      for (long long p = 0; p < N; ++p) {
        const long long gi = c * N + p;
        if (m.pos[p][d] != at || F.h_cmap[gi] != (int)gi) continue;
        double v = F.desc.dirichlet_value[c][b];
        if (A.dfn[f]) {
          double x[3];
          amr_point(m, h->mesh.lower, h->mesh.size, p, x);
          v = A.dfn[f](A.duser[f], f, c, b, x, t);
        }
        F.h_cmap[gi] = -1 - (int)F.h_dvals.size();
        F.h_dvals.push_back(v);
        F.h_drow.push_back(gi);
        any = true;
      }
    }
  F.constrained = any;
  int rc = upload_vec(h, F.cmap, F.h_cmap);
  if (rc) return rc;
  return upload_vec(h, F.dvals, F.h_dvals);
}

// lumped mass with hanging rows condensed onto their masters (deal.II's MatrixFree resolves
// hanging nodes from the mesh in InvMManager::compute_local_scalar, invm_manager.h:173-190)
int build_invm(ppf_handle h) {
  const AmrMesh& m = h->amr->mesh;
  const GLRule g = gauss_lobatto(m.n);
  std::vector<double> jxw(m.N, 0.0);
  for (long long c = 0; c < m.ncells(); ++c) {
    const int lev = m.cells[c].lev;
    double detJ = 1.0;
    for (int d = 0; d < m.dim; ++d) detJ *= level_h(h, d, lev);
    for (int l = 0; l < m.nq; ++l) {
      const int a = l % m.n, b = (l / m.n) % m.n, e = l / (m.n * m.n);
      jxw[m.cell_dofs[(size_t)c * m.nq + l]] += g.w[a] * g.w[b] * (m.dim == 3 ? g.w[e] : 1.0) * detJ;
    }
  }
  for (size_t r = 0; r < m.h_dof.size(); ++r) {
    const int p = m.h_dof[r];
    for (int e = m.h_ptr[r]; e < m.h_ptr[r + 1]; ++e) jxw[m.h_idx[e]] += m.h_w[e] * jxw[p];
  }
  for (size_t r = 0; r < m.h_dof.size(); ++r) jxw[m.h_dof[r]] = 0.0;
  h->h_invm.assign(m.N, 0.0);
  std::vector<double> isq(m.N, 0.0);
  for (long long i = 0; i < m.N; ++i) {
    h->h_invm[i] = jxw[i] == 0.0 ? 0.0 : 1.0 / jxw[i];
    isq[i] = std::sqrt(h->h_invm[i]);
  }
  int rc = upload_vec(h, h->d_invm, h->h_invm);
  if (rc) return rc;
  return upload_vec(h, h->d_invm_sqrt, isq);
}

}  // namespace

// ------------------------------------------------------------------------------------------
// hooks of the runtime
// ------------------------------------------------------------------------------------------
template <int dim, int degree>
static size_t amr_smem_impl(int nlev, int a, int b) {
  return amr_cell_smem_bytes<dim, degree, double>(nlev, a, b);
}

static size_t amr_smem(int dim, int degree, int nlev, int a, int b) {
  switch (dim * 10 + degree) {
    case 21: return amr_smem_impl<2, 1>(nlev, a, b);
    case 22: return amr_smem_impl<2, 2>(nlev, a, b);
    case 31: return amr_smem_impl<3, 1>(nlev, a, b);
    case 32: return amr_smem_impl<3, 2>(nlev, a, b);
    default: return 0;
  }
}

int amr_launch_cell(ppf_handle h, int b, int which, const CellLaunch& L) {
  AmrState& S = *h->amr;
  AmrCellLaunch A;
  std::memset(&A, 0, sizeof(A));
  A.base = L;
  A.base.tables = S.d_tables[2 * b + which];
  if (!A.base.tables) return fail(h, PPF_ERR_ARG, "block has no plan for this operator");
  A.cell_dofs = S.d_cell_dofs;
  A.cell_info = S.d_cell_info;
  A.nlev = S.nlev;
  A.h_ptr = S.d_h_ptr;
  A.h_idx = S.d_h_idx;
  A.h_w = S.d_h_w;
  const BlockPlan& P = h->blocks[b].plan[which];
  const size_t smem = amr_smem(h->dim, h->k, S.nlev, P.nrows_in, P.nrows_out);
  return timed_cell_launch(h, 0, (which == 1 ? MODE_LHS : MODE_RHS) | MODE_AMR, A.base, h->model_obj.data(), smem);
}

static int distribute(ppf_handle h, FieldState& F, double* v) {
  AmrState& S = *h->amr;
  if (!F.h_dvals.empty()) {
    amr_dirichlet_kernel<<<grid_for(F.len), 256, 0, h->stream>>>(v, F.cmap, F.dvals, F.len);
    PPF_CUDA(h, cudaGetLastError());
    h->all_launches++;
  }
  if (S.nrows > 0) {
    dim3 grid(grid_for(S.nrows), F.ncomp);
    amr_hanging_kernel<<<grid, 256, 0, h->stream>>>(v, S.d_h_dof, S.d_h_ptr, S.d_h_idx, S.d_h_w, S.nrows, h->N);
    PPF_CUDA(h, cudaGetLastError());
    h->all_launches++;
  }
  return PPF_OK;
}

int amr_apply_constraints(ppf_handle h, FieldState& F, double* v) { return distribute(h, F, v); }

int amr_finalize_explicit(ppf_handle h, FieldState& F) {
  AmrState& S = *h->amr;
  dim3 grid(grid_for(h->N), F.ncomp);
  amr_finalize_kernel<<<grid, 256, 0, h->stream>>>(F.cur, F.acc, h->d_invm, F.constrained ? F.cmap : nullptr, F.dvals,
                                                   S.d_h_ptr, S.d_h_idx, S.d_h_w, h->N, h->d_err);
  PPF_CUDA(h, cudaGetLastError());
  h->all_launches++;
  return PPF_OK;
}

void amr_fill_hanging(ppf_handle h, int ncomp, double* v) {
  const AmrMesh& m = h->amr->mesh;
  for (int c = 0; c < ncomp; ++c)
    for (size_t r = 0; r < m.h_dof.size(); ++r) {
      double s = 0.0;
      for (int e = m.h_ptr[r]; e < m.h_ptr[r + 1]; ++e) s += m.h_w[e] * v[c * m.N + m.h_idx[e]];
      v[c * m.N + m.h_dof[r]] = s;
    }
}

// the first increment at or after `inc` whose remeshing step runs (UINT_MAX: none)
unsigned amr_next_remesh(ppf_handle h, unsigned inc) {
  const AmrState& S = *h->amr;
  if (inc == 0) return 0;
  if (S.period <= 0) return ~0u;
  const unsigned p = (unsigned)S.period;
  const unsigned long long next = ((unsigned long long)inc + p - 1) / p * p;
  return next > 0xfffffffeULL ? ~0u : (unsigned)next;
}

int amr_permute_io(ppf_handle h, int f, double* host, const double* dev_src, double* dev_dst, int ordering,
                   bool upload) {
  AmrState& S = *h->amr;
  FieldState& F = h->fields[f];
  if (ordering == PPF_ORDER_NATIVE) {
    if (upload) PPF_CUDA(h, cudaMemcpyAsync(dev_dst, host, sizeof(double) * F.len, cudaMemcpyHostToDevice, h->stream));
    else PPF_CUDA(h, cudaMemcpyAsync(host, dev_src, sizeof(double) * F.len, cudaMemcpyDeviceToHost, h->stream));
    PPF_CUDA(h, cudaStreamSynchronize(h->stream));
    return PPF_OK;
  }
  if (ordering != PPF_ORDER_LATTICE || h->mesh_version > 0)
    return fail(h, PPF_ERR_UNSUPPORTED,
                "adaptive meshes exchange vectors in PPF_ORDER_NATIVE (lattice order only before the first remesh)");
  // the initial uniform mesh: lattice node (I,J,K) is the DoF at position (I,J,K) 2^(M-g)
  const AmrMesh& m = S.mesh;
  const int shift = S.max_level - S.global_level;
  const long long nlat = (long long)h->nn[0] * h->nn[1] * h->nn[2];
  std::vector<double> nat(F.len);
  if (!upload) {
    PPF_CUDA(h, cudaMemcpyAsync(nat.data(), dev_src, sizeof(double) * F.len, cudaMemcpyDeviceToHost, h->stream));
    PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  for (long long K = 0; K < h->nn[2]; ++K)
    for (long long J = 0; J < h->nn[1]; ++J)
      for (long long I = 0; I < h->nn[0]; ++I) {
        const long long lat = (K * h->nn[1] + J) * h->nn[0] + I;
        std::array<long long, 3> p{I << shift, J << shift, K << shift};
        for (int d = 0; d < h->dim; ++d)
          if (m.periodic[d] && p[d] == m.E[d]) p[d] = 0;
        if (h->dim < 3) p[2] = 0;
        const int dof = m.node_of.find(m.pos_key(p));
        if (dof < 0) return fail(h, PPF_ERR_CUDA, "internal: lattice node without a DoF");
        // a periodic image reads its master on download; on upload the master's value is kept
        const bool image = (p[0] != (I << shift)) || (p[1] != (J << shift)) || (h->dim == 3 && p[2] != (K << shift));
        for (int c = 0; c < F.ncomp; ++c) {
          if (upload) {
            if (!image) nat[c * m.N + dof] = host[c * nlat + lat];
          } else {
            host[c * nlat + lat] = nat[c * m.N + dof];
          }
        }
      }
  if (upload) {
    PPF_CUDA(h, cudaMemcpyAsync(dev_dst, nat.data(), sizeof(double) * F.len, cudaMemcpyHostToDevice, h->stream));
    PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return PPF_OK;
}

// one remeshing pass (RefinementManager::do_adaptive_refinement + refine_grid,
// refinement_manager.cc:42-87, 393-436)
static int adapt(ppf_handle h) {
  AmrState& S = *h->amr;
  AmrMesh& m = S.mesh;
  using clock = std::chrono::steady_clock;
  auto t_last = clock::now();
  auto lap = [&](int i) {
    const auto t = clock::now();
    S.phase_ms[i] = std::chrono::duration<double, std::milli>(t - t_last).count();
    t_last = t;
  };
  for (double& v : S.phase_ms) v = 0.0;
  // criteria on every cell
  MarkArgs M;
  std::memset(&M, 0, sizeof(M));
  M.ncrit = (int)S.crit.size();
  for (int k = 0; k < M.ncrit; ++k) {
    const FieldState& F = h->fields[S.crit[k].field];
    M.u[k] = F.cur;
    M.ncomp[k] = F.ncomp;
    M.flags[k] = S.crit[k].flags;
    M.vlo[k] = S.crit[k].vlo;
    M.vhi[k] = S.crit[k].vhi;
    M.glo[k] = S.crit[k].glo;
  }
  const GLRule g = gauss_lobatto(m.n);
  for (int i = 0; i < m.n; ++i)
    for (int j = 0; j < m.n; ++j) M.D[i][j] = g.D[i][j];
  for (int l = 0; l < S.nlev; ++l)
    for (int d = 0; d < 3; ++d) M.h[l][d] = d < h->dim ? level_h(h, d, S.min_level + l) : 1.0;
  M.dim = h->dim;
  M.n = m.n;
  M.nq = m.nq;
  M.min_level = S.min_level;
  M.max_level = S.max_level;
  M.N = m.N;
  M.ncells = m.ncells();
  amr_mark_kernel<<<grid_for(m.ncells()), 256, 0, h->stream>>>(M, S.d_cell_dofs, S.d_cell_info, S.d_flags);
  PPF_CUDA(h, cudaGetLastError());
  h->all_launches++;
  std::vector<signed char> flags(m.ncells());
  PPF_CUDA(h, cudaMemcpyAsync(flags.data(), S.d_flags, flags.size(), cudaMemcpyDeviceToHost, h->stream));
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  lap(0);
  amr_smooth(m, flags, S.max_level);
  lap(1);
  bool change = false;
  for (signed char f : flags) change |= f != 0;
  if (!change) {
    // nothing to refine or coarsen: the transfer is the identity, constraints are re-applied
    for (auto& F : h->fields) {
      int rc = distribute(h, F, F.cur);
      for (int a = 0; a < F.n_old && !rc; ++a) rc = distribute(h, F, F.old[a]);
      if (rc) return rc;
    }
    return PPF_OK;
  }
  AmrMesh nm;
  nm.dim = m.dim;
  nm.k = m.k;
  nm.n = m.n;
  nm.nq = m.nq;
  nm.maxlev = m.maxlev;
  for (int d = 0; d < 3; ++d) {
    nm.sub[d] = m.sub[d];
    nm.periodic[d] = m.periodic[d];
    nm.E[d] = m.E[d];
  }
  amr_set_cells(nm, amr_refine(m, flags));
  amr_build(nm);
  std::vector<int> tptr, tidx;
  std::vector<double> tw;
  amr_transfer_plan(m, nm, tptr, tidx, tw);
  lap(2);
  int* d_ptr = nullptr;
  int* d_idx = nullptr;
  double* d_w = nullptr;
  int rc = upload_vec(h, d_ptr, tptr);
  if (!rc) rc = upload_vec(h, d_idx, tidx);
  if (!rc) rc = upload_vec(h, d_w, tw);
  const long long No = m.N, Nn = nm.N;
  // transfer every stored age into vectors of the new length
  for (auto& F : h->fields) {
    if (rc) break;
    const long long len = F.ncomp * Nn;
    double* vecs[5] = {F.cur, F.old[0], F.old[1], F.old[2], F.old[3]};
    for (int a = 0; a <= F.n_old && !rc; ++a) {
      double* nv = nullptr;
      if (cudaMalloc(&nv, sizeof(double) * len) != cudaSuccess) {
        rc = fail(h, PPF_ERR_CUDA, "out of device memory in a remesh");
        break;
      }
      dim3 grid(grid_for(Nn), F.ncomp);
      amr_transfer_kernel<<<grid, 256, 0, h->stream>>>(d_ptr, d_idx, d_w, vecs[a], nv, Nn, No);
      if (cudaGetLastError() != cudaSuccess) rc = fail(h, PPF_ERR_CUDA, "transfer kernel launch");
      h->all_launches++;
      PPF_CUDA(h, cudaStreamSynchronize(h->stream));
      cudaFree(vecs[a]);
      if (a == 0) F.cur = nv;
      else F.old[a - 1] = nv;
    }
    if (rc) break;
    cudaFree(F.acc);
    F.acc = nullptr;
    F.len = len;
    if (cudaMalloc(&F.acc, sizeof(double) * len) != cudaSuccess) rc = fail(h, PPF_ERR_CUDA, "out of device memory");
  }
  cudaFree(d_ptr);
  cudaFree(d_idx);
  cudaFree(d_w);
  if (rc) return rc;
  lap(3);
  m = std::move(nm);
  if ((rc = upload_mesh(h))) return rc;
  if ((rc = build_invm(h))) return rc;
  for (int f = 0; f < (int)h->fields.size(); ++f) {
    FieldState& F = h->fields[f];
    if ((rc = build_constraints(h, f))) return rc;
    if ((rc = distribute(h, F, F.cur))) return rc;
    for (int a = 0; a < F.n_old; ++a)
      if ((rc = distribute(h, F, F.old[a]))) return rc;
  }
  // the host-path scratch of ppf_apply is sized for the old mesh
  cudaFree(h->d_scratch_src);
  cudaFree(h->d_scratch_dst);
  h->d_scratch_src = h->d_scratch_dst = nullptr;
  h->scratch_len = 0;
  h->mesh_version++;
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  lap(4);
  return PPF_OK;
}

// the refinement step of Problem::solve_increment (problem.cc:488-499; initial refinement,
// refinement_manager.cc:104-158)
int amr_remesh_if_due(ppf_handle h) {
  AmrState& S = *h->amr;
  const unsigned inc = h->timer.get_increment();
  if (inc == 0) {
    for (int r = 0; r < S.max_level - S.min_level; ++r) {
      const long long n0 = S.mesh.N;
      int rc = adapt(h);
      if (rc) return rc;
      if (S.mesh.N == n0) break;
    }
  } else if (S.period > 0 && inc % (unsigned)S.period == 0) {
    return adapt(h);
  }
  return PPF_OK;
}

void free_amr(AmrState* A) {
  if (!A) return;
  for (void* p : A->d_tables) cudaFree(p);
  cudaFree(A->d_cell_dofs);
  cudaFree(A->d_cell_info);
  cudaFree(A->d_h_dof);
  cudaFree(A->d_h_ptr);
  cudaFree(A->d_h_idx);
  cudaFree(A->d_h_w);
  cudaFree(A->d_flags);
  delete A;
}

}  // namespace ppf

using namespace ppf;

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------
extern "C" {

int ppf_set_adaptivity(ppf_handle h, const ppf_adaptivity* a) {
  if (!h || !a) return PPF_ERR_ARG;
  if (h->amr) return fail(h, PPF_ERR_ARG, "the mesh is already adaptive");
  if (h->k > 2) return fail(h, PPF_ERR_UNSUPPORTED, "adaptive meshes need degree 1 or 2");
  const int g = h->mesh.global_refinement;
  if (a->min_refinement < 0 || a->min_refinement > g || a->max_refinement < g ||
      a->max_refinement - a->min_refinement + 1 > AMR_MAX_LEVELS)
    return fail(h, PPF_ERR_ARG, "refinement levels: need min <= global refinement <= max");
  if (a->n_criteria < 0 || a->n_criteria > PPF_MAX_FIELDS) return PPF_ERR_ARG;
  for (int d = 0; d < h->dim; ++d)
    if (h->mesh.periodic[d] && ((long long)h->mesh.subdivisions[d] << a->min_refinement) < 2)
      return fail(h, PPF_ERR_UNSUPPORTED, "a periodic direction needs two cells at the minimum refinement");
  std::unique_ptr<AmrState> S(new AmrState());
  S->min_level = a->min_refinement;
  S->max_level = a->max_refinement;
  S->period = a->remeshing_period;
  S->global_level = g;
  S->nlev = S->max_level - S->min_level + 1;
  for (int i = 0; i < a->n_criteria; ++i) {
    const int f = a->criterion_field[i];
    if (f < 0 || f >= (int)h->fields.size()) return fail(h, PPF_ERR_ARG, "refinement criterion on an unknown field");
    S->crit.push_back({f, a->criterion_flags[i], a->value_lower[i], a->value_upper[i], a->gradient_lower[i]});
  }
  S->dfn.assign(h->fields.size(), nullptr);
  S->duser.assign(h->fields.size(), nullptr);
  std::string err;
  if (!amr_init_uniform(S->mesh, h->dim, h->k, h->mesh.subdivisions, h->mesh.periodic, g, S->max_level, err))
    return fail(h, PPF_ERR_UNSUPPORTED, err);
  amr_build(S->mesh);
  // per-level cell tables of every plan
  S->d_tables.assign(2 * h->blocks.size(), nullptr);
  for (size_t b = 0; b < h->blocks.size(); ++b)
    for (int which = 0; which < 2; ++which) {
      const BlockPlan& P = h->blocks[b].plan[which];
      if (!P.valid) continue;
      std::vector<unsigned char> all;
      for (int l = S->min_level; l <= S->max_level; ++l) {
        double hl[3] = {1.0, 1.0, 1.0};
        for (int d = 0; d < h->dim; ++d) hl[d] = level_h(h, d, l);
        auto t = build_cell_tables(h->dim, h->k, 0, h->mesh.lower, hl, P.slot_of, P.slot_comp0, P.out_of, P.out_row0);
        if (t.empty()) return fail(h, PPF_ERR_UNSUPPORTED, "unsupported dim/degree");
        all.insert(all.end(), t.begin(), t.end());
      }
      void* d = nullptr;
      PPF_CUDA(h, cudaMalloc(&d, all.size()));
      PPF_CUDA(h, cudaMemcpyAsync(d, all.data(), all.size(), cudaMemcpyHostToDevice, h->stream));
      PPF_CUDA(h, cudaStreamSynchronize(h->stream));
      S->d_tables[2 * b + which] = d;
    }
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  h->amr = S.release();
  int rc = upload_mesh(h);
  if (rc) return rc;
  // field states on the adaptive numbering of the initial mesh (zeroed)
  for (int f = 0; f < (int)h->fields.size(); ++f) {
    FieldState& F = h->fields[f];
    cudaFree(F.cur);
    for (int k = 0; k < 4; ++k) {
      cudaFree(F.old[k]);
      F.old[k] = nullptr;
    }
    cudaFree(F.acc);
    F.len = F.ncomp * h->N;
    PPF_CUDA(h, cudaMalloc(&F.cur, sizeof(double) * F.len));
    PPF_CUDA(h, cudaMemsetAsync(F.cur, 0, sizeof(double) * F.len, h->stream));
    for (int k = 0; k < F.n_old; ++k) {
      PPF_CUDA(h, cudaMalloc(&F.old[k], sizeof(double) * F.len));
      PPF_CUDA(h, cudaMemsetAsync(F.old[k], 0, sizeof(double) * F.len, h->stream));
    }
    PPF_CUDA(h, cudaMalloc(&F.acc, sizeof(double) * F.len));
    if ((rc = build_constraints(h, f))) return rc;
  }
  if ((rc = build_invm(h))) return rc;
  if (h->run_graph) {
    cudaGraphExecDestroy(h->run_graph);
    h->run_graph = nullptr;
  }
  cudaFree(h->d_scratch_src);
  cudaFree(h->d_scratch_dst);
  h->d_scratch_src = h->d_scratch_dst = nullptr;
  h->scratch_len = 0;
  h->mesh_version = 0;
  return PPF_OK;
}

int ppf_adapt(ppf_handle h) {
  if (!h) return PPF_ERR_ARG;
  if (!h->amr) return fail(h, PPF_ERR_ARG, "the mesh is not adaptive");
  int rc = adapt(h);
  if (rc) return rc;
  return check_err(h);
}

int ppf_remesh_if_due(ppf_handle h) {
  if (!h) return PPF_ERR_ARG;
  if (!h->amr) return PPF_OK;
  int rc = amr_remesh_if_due(h);
  if (rc) return rc;
  return check_err(h);
}

long long ppf_mesh_version(ppf_handle h) { return h ? h->mesh_version : -1; }

int ppf_remesh_stats(ppf_handle h, double* phases_ms) {
  if (!h || !phases_ms) return PPF_ERR_ARG;
  if (!h->amr) return fail(h, PPF_ERR_ARG, "the mesh is not adaptive");
  for (int i = 0; i < 5; ++i) phases_ms[i] = h->amr->phase_ms[i];
  return PPF_OK;
}

int ppf_cells(ppf_handle h, int* out) {
  if (!h || !out) return PPF_ERR_ARG;
  if (h->amr) {
    const AmrMesh& m = h->amr->mesh;
    for (long long c = 0; c < m.ncells(); ++c) {
      out[4 * c] = m.cells[c].lev;
      for (int d = 0; d < 3; ++d) out[4 * c + 1 + d] = m.cells[c].x[d];
    }
    return PPF_OK;
  }
  for (long long c = 0; c < h->ncells; ++c) {
    out[4 * c] = h->mesh.global_refinement;
    out[4 * c + 1] = (int)(c % h->nc[0]);
    out[4 * c + 2] = (int)((c / h->nc[0]) % h->nc[1]);
    out[4 * c + 3] = (int)(c / ((long long)h->nc[0] * h->nc[1]));
  }
  return PPF_OK;
}

int ppf_cell_dofs(ppf_handle h, int* out) {
  if (!h || !out) return PPF_ERR_ARG;
  if (h->amr) {
    std::memcpy(out, h->amr->mesh.cell_dofs.data(), sizeof(int) * h->amr->mesh.cell_dofs.size());
    return PPF_OK;
  }
  const int n = h->n, k = h->k, nq = h->dim == 2 ? n * n : n * n * n;
  for (long long c = 0; c < h->ncells; ++c) {
    const long long cx = c % h->nc[0], cy = (c / h->nc[0]) % h->nc[1], cz = c / ((long long)h->nc[0] * h->nc[1]);
    for (int q = 0; q < nq; ++q) {
      const int a = q % n, b = (q / n) % n, e = h->dim == 3 ? q / (n * n) : 0;
      out[c * nq + q] = (int)(((k * cz + e) * h->nn[1] + (k * cy + b)) * h->nn[0] + (k * cx + a));
    }
  }
  return PPF_OK;
}

int ppf_node_points(ppf_handle h, double* out) {
  if (!h || !out) return PPF_ERR_ARG;
  if (h->amr) {
    for (long long p = 0; p < h->amr->mesh.N; ++p) amr_point(h->amr->mesh, h->mesh.lower, h->mesh.size, p, out + 3 * p);
    return PPF_OK;
  }
  const GLRule g = gauss_lobatto(h->n);
  for (long long i = 0; i < h->N; ++i) {
    const long long I[3] = {i % h->nn[0], (i / h->nn[0]) % h->nn[1], i / ((long long)h->nn[0] * h->nn[1])};
    for (int d = 0; d < 3; ++d) {
      if (d >= h->dim) {
        out[3 * i + d] = 0.0;
        continue;
      }
      const long long cell = std::min<long long>(I[d] / h->k, h->nc[d] - 1);
      out[3 * i + d] = h->mesh.lower[d] + (cell + g.x[I[d] - cell * h->k]) * h->h[d];
    }
  }
  return PPF_OK;
}

long long ppf_hanging(ppf_handle h, int* count, int* master, double* weight) {
  if (!h) return -1;
  if (!h->amr) {
    if (count) std::memset(count, 0, sizeof(int) * h->N);
    return 0;
  }
  const AmrMesh& m = h->amr->mesh;
  if (count)
    for (long long p = 0; p < m.N; ++p) {
      const int r = m.hang_row[p];
      count[p] = r < 0 ? 0 : m.h_ptr[r + 1] - m.h_ptr[r];
    }
  if (master) std::memcpy(master, m.h_idx.data(), sizeof(int) * m.h_idx.size());
  if (weight) std::memcpy(weight, m.h_w.data(), sizeof(double) * m.h_w.size());
  return (long long)m.h_idx.size();
}

int ppf_set_dirichlet_function(ppf_handle h, int f, ppf_dirichlet_fn fn, void* user) {
  if (!h || f < 0 || f >= (int)h->fields.size()) return PPF_ERR_ARG;
  if (!h->amr) return fail(h, PPF_ERR_UNSUPPORTED, "Dirichlet functions are for adaptive meshes (use ppf_set_dirichlet_values)");
  h->amr->dfn[f] = fn;
  h->amr->duser[f] = user;
  int rc = build_constraints(h, f);
  if (rc) return rc;
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  return PPF_OK;
}

}  // extern "C"
