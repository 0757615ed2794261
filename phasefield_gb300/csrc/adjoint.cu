// Adjoint of the explicit coupled Allen-Cahn / Cahn-Hilliard step with binomial
// checkpointing, and its tangent-linear reference.
//
// The explicit step u+ = F(u) = invM (.) R(u; theta) (ExplicitSolver::solve_impl,
// include/prismspf/solvers/explicit_solver.h:63-77, with the coupled application's block 0,
// applications/coupled_allen_cahn_cahn_hilliard/custom_pde.h:63-139) is reversed step by step:
//   lambda_k = (dF/du(u_k))^T lambda_{k+1} = (dR/du)^T (invM (.) lambda_{k+1})
//   dJ/dtheta += (dR/dtheta)^T (invM (.) lambda_{k+1})
// both computed by the cell kernel with the CoupledACCHAdjoint operator (transposed
// sum-factorised apply with the pointwise Jacobians). The trajectory is not stored: with S
// snapshot slots a step k is recomputed from the nearest snapshot, the snapshots placed by the
// binomial rule of Griewank's revolve (for n steps and s free slots, t the smallest repetition
// number with C(s+t, s) >= n, the first checkpoint goes n - C(s-1+t, s-1) steps ahead), so each
// step is recomputed at most t times. The forward call leaves the first checkpoints of that
// schedule in place.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "handle.h"
#include "models.cuh"

namespace ppf {

struct AdjointState {
  int block = -1;
  int K = 0;
  int S = 0;                     // snapshot slots (u_0 included)
  long long N = 0;
  std::vector<double*> slot;     // S + 1 slots (the last one is a work slot), 2N each
  std::vector<int> slot_step;    // step stored in a slot, -1 when free
  double* lam = nullptr;         // 2N
  double* lam_new = nullptr;     // 2N accumulator
  double* w = nullptr;           // 2N: invM (.) lambda
  double* gpar = nullptr;        // 2N: dMc, dKn densities (accumulated over all steps)
  double* du = nullptr;          // 2N tangent state
  double* dacc = nullptr;        // 2N tangent accumulator
  void* tab = nullptr;           // cell tables of the linearised operators
  std::vector<unsigned char> obj_adj;
  long long forward_steps = 0;
  bool ready = false;
};

namespace {

__global__ void scale_by_invm_kernel(double* __restrict__ out, const double* __restrict__ in,
                                     const double* __restrict__ invm, long long N, int nf) {
  const long long total = N * nf;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    out[i] = in[i] * invm[i % N];
}

long long binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  long double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return (long long)(r + 0.5);
}

// steps to advance before the next checkpoint when n steps are reversed with s free slots
int split(int n, int s) {
  if (s <= 0 || n <= 1) return 1;
  int t = 0;
  while (binom(s + t, s) < n) ++t;
  const long long m = (long long)n - binom(s - 1 + t, s - 1);
  return (int)std::max<long long>(1, std::min<long long>(m, n - 1));
}

int slot_of_step(AdjointState& A, int step) {
  for (size_t i = 0; i < A.slot_step.size(); ++i)
    if (A.slot_step[i] == step) return (int)i;
  return -1;
}

int free_slot(AdjointState& A) {
  for (int i = 0; i < A.S; ++i)
    if (A.slot_step[i] < 0) return i;
  return -1;
}

struct Fields {
  FieldState* c;
  FieldState* n;
};

Fields block_fields(ppf_handle h, int b) {
  const ppf_block_desc& d = h->blocks[b].desc;
  return {&h->fields[d.field_indices[0]], &h->fields[d.field_indices[1]]};
}

// state (2N) -> old_1 of the block fields, one explicit solve, result -> dst (2N)
int forward_step(ppf_handle h, AdjointState& A, const double* src, double* dst) {
  Fields f = block_fields(h, A.block);
  const size_t bytes = sizeof(double) * A.N;
  PPF_CUDA(h, cudaMemcpyAsync(f.c->old[0], src, bytes, cudaMemcpyDeviceToDevice, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(f.n->old[0], src + A.N, bytes, cudaMemcpyDeviceToDevice, h->stream));
  int rc = explicit_solve_entry(h, A.block);
  if (rc) return rc;
  PPF_CUDA(h, cudaMemcpyAsync(dst, f.c->cur, bytes, cudaMemcpyDeviceToDevice, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(dst + A.N, f.n->cur, bytes, cudaMemcpyDeviceToDevice, h->stream));
  A.forward_steps++;
  return PPF_OK;
}

// u_m from the snapshot of step a, stored in slot `dst`
int advance(ppf_handle h, AdjointState& A, int a, int m, int dst) {
  const int src = slot_of_step(A, a);
  if (src < 0) return fail(h, PPF_ERR_ARG, "internal: missing checkpoint");
  double* work = A.slot[A.S];
  const double* cur = A.slot[src];
  for (int k = a; k < m; ++k) {
    double* out = (k + 1 == m) ? A.slot[dst] : work;  // in place on the work slot is fine
    int rc = forward_step(h, A, cur, out);
    if (rc) return rc;
    cur = out;
  }
  if (cur != A.slot[dst])
    PPF_CUDA(h, cudaMemcpyAsync(A.slot[dst], cur, sizeof(double) * 2 * A.N, cudaMemcpyDeviceToDevice, h->stream));
  A.slot_step[dst] = m;
  return PPF_OK;
}

// cell launch of a linearised operator: inputs u (2 fields at Current) and dir (2 fields at
// SRC), outputs `nout` accumulators
int linearised_launch(ppf_handle h, AdjointState& A, const char* model, const void* obj, const double* u,
                      const double* dir, double* const* outs, int nout) {
  const ModelOps* ops = find_model(model);
  if (!ops) return fail(h, PPF_ERR_UNSUPPORTED, "linearised operator set not compiled in");
  CellLaunch L;
  std::memset(&L, 0, sizeof(L));
  for (int d = 0; d < 3; ++d) {
    L.nc[d] = h->nc[d];
    L.nn[d] = h->nn[d];
  }
  L.N = h->N;
  L.ncells = h->ncells;
  L.nslots = 4;
  const double* ptrs[4] = {u, u + A.N, dir, dir + A.N};
  for (int s = 0; s < 4; ++s) {
    L.slots[s].ptr = ptrs[s];
    L.slots[s].ncomp = 1;
  }
  L.nout = nout;
  for (int o = 0; o < nout; ++o) {
    L.outs[o].acc = outs[o];
    L.outs[o].ncomp = 1;
  }
  L.nrows_in = 4;
  L.nrows_out = 4 * (1 + h->dim);
  L.tables = A.tab;
  L.timer = h->timer;
  L.block_id = 0;
  L.err = h->d_err;
  L.fx_deriv = 1;  // integer derivatives where the tables allow them (FP64 Q1/Q2)
  const size_t smem = cell_smem(h->dim, h->k, 0, L.nrows_in, L.nrows_out);
  cudaError_t e = ops->launch(h->dim, h->k, MODE_RHS, 0, L, obj, smem, h->stream);
  if (e != cudaSuccess) return fail(h, PPF_ERR_CUDA, std::string("linearised kernel: ") + cudaGetErrorString(e));
  h->cell_launches++;
  h->all_launches++;
  return PPF_OK;
}

// lambda_a from lambda_{a+1} with the state u_a; parameter densities accumulate in gpar
int adjoint_step(ppf_handle h, AdjointState& A, int a) {
  const int s = slot_of_step(A, a);
  if (s < 0) return fail(h, PPF_ERR_ARG, "internal: adjoint step without its state");
  scale_by_invm_kernel<<<grid_for(2 * A.N), 256, 0, h->stream>>>(A.w, A.lam, h->d_invm, A.N, 2);
  PPF_CUDA(h, cudaMemsetAsync(A.lam_new, 0, sizeof(double) * 2 * A.N, h->stream));
  double* outs[4] = {A.lam_new, A.lam_new + A.N, A.gpar, A.gpar + A.N};
  int rc = linearised_launch(h, A, "coupled_acch_adjoint", A.obj_adj.data(), A.slot[s], A.w, outs, 4);
  if (rc) return rc;
  std::swap(A.lam, A.lam_new);
  return PPF_OK;
}

int reverse(ppf_handle h, AdjointState& A, int a, int b, int s) {
  if (b - a == 1) return adjoint_step(h, A, a);
  if (s <= 0) {  // no free slot: recompute each state from a in the work slot
    for (int j = b - 1; j >= a; --j) {
      if (j == a) {
        int rc = adjoint_step(h, A, a);
        if (rc) return rc;
        continue;
      }
      // the work slot doubles as the state of step j
      const int src = slot_of_step(A, a);
      double* work = A.slot[A.S];
      PPF_CUDA(h, cudaMemcpyAsync(work, A.slot[src], sizeof(double) * 2 * A.N, cudaMemcpyDeviceToDevice, h->stream));
      for (int k = a; k < j; ++k) {
        int rc = forward_step(h, A, work, work);
        if (rc) return rc;
      }
      A.slot_step[A.S] = j;
      int rc = adjoint_step(h, A, j);
      A.slot_step[A.S] = -1;
      if (rc) return rc;
    }
    return PPF_OK;
  }
  const int m = a + split(b - a, s);
  int sm = slot_of_step(A, m);
  bool stored_here = false;
  if (sm < 0) {
    sm = free_slot(A);
    if (sm < 0) return fail(h, PPF_ERR_ARG, "internal: no free checkpoint slot");
    int rc = advance(h, A, a, m, sm);
    if (rc) return rc;
    stored_here = true;
  }
  (void)stored_here;
  int rc = reverse(h, A, m, b, s - 1);
  if (rc) return rc;
  A.slot_step[sm] = -1;
  return reverse(h, A, a, m, s);
}

int check_block(ppf_handle h, int b) {
  if (b < 0 || b >= (int)h->blocks.size()) return fail(h, PPF_ERR_ARG, "bad block");
  if (h->amr) return fail(h, PPF_ERR_UNSUPPORTED, "the adjoint runs on uniform meshes");
  const ppf_block_desc& d = h->blocks[b].desc;
  if (std::strcmp(h->model->name, "coupled_acch") != 0 || d.n_fields != 2 || d.solve_type != PPF_EXPLICIT)
    return fail(h, PPF_ERR_UNSUPPORTED, "the adjoint is implemented for the coupled_acch explicit block");
  for (int i = 0; i < 2; ++i) {
    const FieldState& F = h->fields[d.field_indices[i]];
    if (F.rank != 0 || F.constrained)
      return fail(h, PPF_ERR_UNSUPPORTED, "adjoint: scalar fields without constraints only");
    if (F.n_old < 1) return fail(h, PPF_ERR_ARG, "adjoint: block must depend on old_1 of its fields");
  }
  return PPF_OK;
}

int setup(ppf_handle h, AdjointState& A, int b, int S) {
  A.block = b;
  A.S = std::max(1, S);
  A.N = h->N;
  for (double* p : A.slot) cudaFree(p);
  A.slot.assign(A.S + 1, nullptr);
  A.slot_step.assign(A.S + 1, -1);
  for (auto& p : A.slot) PPF_CUDA(h, cudaMalloc(&p, sizeof(double) * 2 * A.N));
  if (!A.lam) {
    for (double** p : {&A.lam, &A.lam_new, &A.w, &A.gpar, &A.du, &A.dacc})
      PPF_CUDA(h, cudaMalloc(p, sizeof(double) * 2 * A.N));
    signed char slot_of[pg::MAX_FIELDS][pg::NAGE];
    signed char slot_comp0[pg::MAX_SLOTS] = {0, 1, 2, 3};
    signed char out_of[pg::MAX_FIELDS];
    signed char out_row0[pg::MAX_OUTS];
    std::memset(slot_of, -1, sizeof(slot_of));
    std::memset(out_of, -1, sizeof(out_of));
    slot_of[0][0] = 0;
    slot_of[1][0] = 1;
    slot_of[0][5] = 2;
    slot_of[1][5] = 3;
    for (int o = 0; o < 4; ++o) {
      out_of[o] = (signed char)o;
      out_row0[o] = (signed char)(o * (1 + h->dim));
    }
    double lo[3] = {h->mesh.lower[0], h->mesh.lower[1], h->mesh.lower[2]};
    auto tab = build_cell_tables(h->dim, h->k, 0, lo, h->h, slot_of, slot_comp0, out_of, out_row0);
    PPF_CUDA(h, cudaMalloc(&A.tab, tab.size()));
    PPF_CUDA(h, cudaMemcpy(A.tab, tab.data(), tab.size(), cudaMemcpyHostToDevice));
    const ModelOps* ops = find_model("coupled_acch_adjoint");
    if (!ops) return fail(h, PPF_ERR_UNSUPPORTED, "adjoint operator set not compiled in");
    A.obj_adj.resize(256);
    std::string err;
    const size_t sz = ops->make_object(h->dim, h->k, 0, h->constants.data(), (int)h->constants.size(),
                                       A.obj_adj.data(), A.obj_adj.size(), &err);
    if (!sz) return fail(h, PPF_ERR_ARG, err);
    A.obj_adj.resize(sz);
  }
  A.ready = true;
  return PPF_OK;
}

}  // namespace

void free_adjoint(AdjointState* A) {
  if (!A) return;
  for (double* p : A->slot) cudaFree(p);
  for (double* p : {A->lam, A->lam_new, A->w, A->gpar, A->du, A->dacc}) cudaFree(p);
  cudaFree(A->tab);
  delete A;
}

}  // namespace ppf

using namespace ppf;

extern "C" {

int ppf_adjoint_forward(ppf_handle h, int b, int n_steps, int n_snapshots) {
  if (!h || n_steps < 1 || n_snapshots < 1) return PPF_ERR_ARG;
  int rc = check_block(h, b);
  if (rc) return rc;
  if (!h->adj) h->adj = new AdjointState();
  AdjointState& A = *h->adj;
  rc = setup(h, A, b, n_snapshots);
  if (rc) return rc;
  A.K = n_steps;
  A.forward_steps = 0;
  Fields f = block_fields(h, b);
  PPF_CUDA(h, cudaMemcpyAsync(A.slot[0], f.c->cur, sizeof(double) * A.N, cudaMemcpyDeviceToDevice, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(A.slot[0] + A.N, f.n->cur, sizeof(double) * A.N, cudaMemcpyDeviceToDevice, h->stream));
  A.slot_step[0] = 0;
  // first sweep: the chain of first checkpoints of the binomial schedule, then on to n_steps
  int a = 0, s = A.S - 1;
  while (n_steps - a > 1 && s >= 1) {
    const int m = a + split(n_steps - a, s);
    const int slot = free_slot(A);
    rc = advance(h, A, a, m, slot);
    if (rc) return rc;
    a = m;
    --s;
  }
  // u_K into the work slot and the fields' current vectors
  const int src = slot_of_step(A, a);
  double* work = A.slot[A.S];
  PPF_CUDA(h, cudaMemcpyAsync(work, A.slot[src], sizeof(double) * 2 * A.N, cudaMemcpyDeviceToDevice, h->stream));
  for (int k = a; k < n_steps; ++k) {
    rc = forward_step(h, A, work, work);
    if (rc) return rc;
  }
  PPF_CUDA(h, cudaMemcpyAsync(f.c->cur, work, sizeof(double) * A.N, cudaMemcpyDeviceToDevice, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(f.n->cur, work + A.N, sizeof(double) * A.N, cudaMemcpyDeviceToDevice, h->stream));
  return check_err(h);
}

int ppf_adjoint_backward(ppf_handle h, const double* dJ_duK, double* dJ_dparams, double* dJ_du0,
                         long long* forward_steps) {
  if (!h || !h->adj || !h->adj->ready || !dJ_duK) return PPF_ERR_ARG;
  AdjointState& A = *h->adj;
  PPF_CUDA(h, cudaMemcpyAsync(A.lam, dJ_duK, sizeof(double) * 2 * A.N, cudaMemcpyHostToDevice, h->stream));
  PPF_CUDA(h, cudaMemsetAsync(A.gpar, 0, sizeof(double) * 2 * A.N, h->stream));
  int rc = reverse(h, A, 0, A.K, A.S - 1);
  if (rc) return rc;
  std::vector<double> g(2 * A.N);
  PPF_CUDA(h, cudaMemcpyAsync(g.data(), A.gpar, sizeof(double) * 2 * A.N, cudaMemcpyDeviceToHost, h->stream));
  if (dJ_du0) PPF_CUDA(h, cudaMemcpyAsync(dJ_du0, A.lam, sizeof(double) * 2 * A.N, cudaMemcpyDeviceToHost, h->stream));
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  if (dJ_dparams) {
    double s0 = 0.0, s1 = 0.0;
    for (long long i = 0; i < A.N; ++i) {
      s0 += g[i];
      s1 += g[A.N + i];
    }
    dJ_dparams[0] = s0;
    dJ_dparams[1] = s1;
  }
  if (forward_steps) *forward_steps = A.forward_steps;
  // restore the first checkpoints so another backward pass could run; the state is kept
  return check_err(h);
}

// Tangent-linear reference: du_K for a perturbation (du_0, dMc, dKn) from the block fields'
// current state u_0 (host vectors, block fields concatenated); the state is left unchanged.
int ppf_tangent_linear(ppf_handle h, int b, int n_steps, const double* du0, const double* dparams, double* duK) {
  if (!h || n_steps < 0 || !du0 || !dparams || !duK) return PPF_ERR_ARG;
  int rc = check_block(h, b);
  if (rc) return rc;
  if (!h->adj) h->adj = new AdjointState();
  AdjointState& A = *h->adj;
  if (!A.ready || A.block != b) {
    rc = setup(h, A, b, 1);
    if (rc) return rc;
  }
  const ModelOps* ops = find_model("coupled_acch_tangent");
  if (!ops) return fail(h, PPF_ERR_UNSUPPORTED, "tangent operator set not compiled in");
  std::vector<unsigned char> obj(256);
  double cst[5] = {h->constants[0], h->constants[1], h->constants[2], dparams[0], dparams[1]};
  std::string err;
  const size_t sz = ops->make_object(h->dim, h->k, 0, cst, 5, obj.data(), obj.size(), &err);
  if (!sz) return fail(h, PPF_ERR_ARG, err);
  Fields f = block_fields(h, b);
  double* u = A.slot[A.S];  // work slot: the forward state along the way
  PPF_CUDA(h, cudaMemcpyAsync(u, f.c->cur, sizeof(double) * A.N, cudaMemcpyDeviceToDevice, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(u + A.N, f.n->cur, sizeof(double) * A.N, cudaMemcpyDeviceToDevice, h->stream));
  // keep u_0 to restore the fields afterwards
  std::vector<double> u0(2 * A.N);
  PPF_CUDA(h, cudaMemcpyAsync(u0.data(), u, sizeof(double) * 2 * A.N, cudaMemcpyDeviceToHost, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(A.du, du0, sizeof(double) * 2 * A.N, cudaMemcpyHostToDevice, h->stream));
  for (int k = 0; k < n_steps; ++k) {
    PPF_CUDA(h, cudaMemsetAsync(A.dacc, 0, sizeof(double) * 2 * A.N, h->stream));
    double* outs[2] = {A.dacc, A.dacc + A.N};
    rc = linearised_launch(h, A, "coupled_acch_tangent", obj.data(), u, A.du, outs, 2);
    if (rc) return rc;
    scale_by_invm_kernel<<<grid_for(2 * A.N), 256, 0, h->stream>>>(A.du, A.dacc, h->d_invm, A.N, 2);
    rc = forward_step(h, A, u, u);
    if (rc) return rc;
  }
  PPF_CUDA(h, cudaMemcpyAsync(duK, A.du, sizeof(double) * 2 * A.N, cudaMemcpyDeviceToHost, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(f.c->cur, u0.data(), sizeof(double) * A.N, cudaMemcpyHostToDevice, h->stream));
  PPF_CUDA(h, cudaMemcpyAsync(f.n->cur, u0.data() + A.N, sizeof(double) * A.N, cudaMemcpyHostToDevice, h->stream));
  PPF_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_err(h);
}

// Forward recomputation count of the binomial schedule for n steps and S slots (host only).
long long ppf_checkpoint_schedule_cost(int n_steps, int n_snapshots) {
  if (n_steps < 1 || n_snapshots < 1) return -1;
  // simulate reverse(0, n, S-1) counting forward steps; the first sweep advances to n
  struct Sim {
    long long steps = 0;
    void rev(int a, int b, int s, std::vector<int>& have) {
      if (b - a == 1) return;
      if (s <= 0) {
        for (int j = b - 1; j > a; --j) steps += j - a;
        return;
      }
      const int m = a + split(b - a, s);
      if (std::find(have.begin(), have.end(), m) == have.end()) steps += m - a;
      else have.erase(std::find(have.begin(), have.end(), m));
      rev(m, b, s - 1, have);
      rev(a, m, s, have);
    }
  } sim;
  std::vector<int> first;  // checkpoints left by the forward sweep
  int a = 0, s = n_snapshots - 1;
  while (n_steps - a > 1 && s >= 1) {
    a += split(n_steps - a, s);
    first.push_back(a);
    --s;
  }
  sim.rev(0, n_steps, n_snapshots - 1, first);
  return n_steps + sim.steps;
}

}  // extern "C"
