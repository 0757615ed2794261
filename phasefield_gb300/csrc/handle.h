// Internal definition of the engine handle shared by the runtime translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/ppf_gb300.h"
#include "runtime.h"

namespace ppf {

struct GLRule {
  int n;
  double x[pg::MAX_N], w[pg::MAX_N], D[pg::MAX_N][pg::MAX_N];
};
GLRule gauss_lobatto(int n);

struct FieldState {
  int rank = 0, ncomp = 1;
  long long len = 0;
  int n_old = 0;
  double* cur = nullptr;
  double* old[4] = {nullptr, nullptr, nullptr, nullptr};
  double* acc = nullptr;
  int* cmap = nullptr;
  double* dvals = nullptr;
  std::vector<int> h_cmap;
  std::vector<double> h_dvals;
  std::vector<long long> h_drow;  // position (component-major lattice index) of Dirichlet row j
  bool constrained = false;
  ppf_field_desc desc;
  // host destination the field is streamed to after every increment (ppf_set_output_stream)
  double* stream_out = nullptr;
  bool streamed = false;  // copied during the current increment
  // pipelined I/O (ppf_upload_state_staged, ppf_run_async): per age a device staging buffer the
  // upload stream fills ahead of the run that consumes it, with its ready / consumed events
  double* in_stage[5] = {};
  cudaEvent_t in_ready[5] = {};
  cudaEvent_t in_free[5] = {};
  bool in_pending[5] = {};
  // a queued run streams the field out of this copy, so the next increment may overwrite the
  // state while the copy to the host is in flight; out_free marks the end of that copy
  double* out_stage = nullptr;
  cudaEvent_t out_free = nullptr;
};

struct BlockPlan {
  int nslots = 0;
  int slot_field[pg::MAX_SLOTS];
  int slot_age[pg::MAX_SLOTS];
  int nrows_in = 0, nrows_out = 0;
  void* d_tables = nullptr;
  std::vector<unsigned char> h_tables;  // host copy (the lane kernel takes it as a kernel parameter)
  bool valid = false;
  // the slot tables of the plan (host copies; adaptive meshes build one CellTables per level)
  signed char slot_of[pg::MAX_FIELDS][pg::NAGE];
  signed char slot_comp0[pg::MAX_SLOTS];
  signed char out_of[pg::MAX_FIELDS];
  signed char out_row0[pg::MAX_OUTS];
  // integer contractions (FP64 Q1/Q2): on in the tables; arithmetic chosen for this plan
  // (-1 until the first plain launch times the modes; 1 integer derivatives + FP64
  // integration, 2 both in integers, 3 FP64 derivatives + integer integration, 4 the lane kernel:
  // every contraction in integers, cubic cells only)
  bool fx = false;
  bool fx_lanes = false;
  int fx_mode = -1;
  int fx_timed = 0;                // online timing of the multigrid outer operator
  cudaEvent_t fx_ev[16] = {};
  unsigned int fx_rows = 0;        // value rows read as gradients
  unsigned int val_rows = 0;       // value rows read as values or Hessians
};

// One mesh of a multigrid hierarchy for a single-field linear block (the finest level is the
// problem mesh). Vectors are allocated in the level's working precision.
struct MGLevel {
  int refine = 0;
  int nc[3] = {1, 1, 1}, nn[3] = {1, 1, 1};
  double h[3] = {1, 1, 1};
  long long N = 0, ncells = 0, len = 0;
  int precision = 0;            // 0 FP64, 1 FP32
  int* cmap = nullptr;          // homogeneous level constraints
  bool constrained = false;
  void* invm_sqrt = nullptr;    // per node, level precision
  void* inv_diag = nullptr;     // len, level precision
  void* tables = nullptr;       // CellTables for the LHS (level precision)
  std::vector<unsigned char> h_tables;  // host copy (the lane kernel takes it as a kernel parameter)
  bool fx_lanes = false;        // FP64 level whose tables allow the lane kernel
  void* acc = nullptr;          // accumulator
  void* x = nullptr;            // level solution
  void* b = nullptr;            // level defect (right-hand side)
  void* r = nullptr;            // residual / work
  void* w0 = nullptr;           // work vectors
  void* w1 = nullptr;
  double lambda_max = 0.0;      // Chebyshev interval
  double lambda_min = 0.0;
  bool eig_done = false;
  // separable transfer to the next finer level: per axis CSR of the 1-D prolongation
  // (fine index -> coarse entries) and of its transpose (coarse index -> fine entries)
  int* p_ptr[3] = {nullptr, nullptr, nullptr};
  int* p_col[3] = {nullptr, nullptr, nullptr};
  void* p_val[3] = {nullptr, nullptr, nullptr};
  int* r_ptr[3] = {nullptr, nullptr, nullptr};
  int* r_col[3] = {nullptr, nullptr, nullptr};
  void* r_val[3] = {nullptr, nullptr, nullptr};
  void* t0 = nullptr;           // transfer work buffers (fine-sized)
  void* t1 = nullptr;
  void* cvt = nullptr;          // precision-conversion buffer (coarsest level of a mixed hierarchy)
  // contraction mode of the level's FP64 operator (integer contractions, FP64 Q1/Q2): its first
  // plain LHS launches run modes 1, 2, 3 (and 4 where the lane kernel applies) twice under CUDA
  // events, then the fastest stays
  int fx_mode = -1;
  int fx_timed = 0;
  cudaEvent_t fx_ev[16] = {};
};

struct AdjointState;
struct AmrState;

struct LinearState {
  ppf_linear_params params;
  bool params_set = false;
  bool initialized = false;
  std::vector<MGLevel> levels;  // coarse .. fine
  double* rhs = nullptr;        // FP64 fine vectors
  double* g = nullptr;          // inhomogeneous values
  double* x_hom = nullptr;      // homogeneous solution (next initial guess)
  double* r = nullptr;
  double* p = nullptr;
  double* q = nullptr;
  double* z = nullptr;
  double* inv_diag = nullptr;   // fine FP64 inverse diagonal (Chebyshev preconditioner)
  double* partial = nullptr;    // dot-product partial sums
  double cheb_lmax = 0.0, cheb_lmin = 0.0;
  bool cheb_eig_done = false;
  int last_iterations = 0;
  double last_residual = 0.0;
  double last_rhs_norm = 0.0;
  // the preconditioner application captured as a CUDA graph (rebuilt for every solve)
  cudaGraphExec_t pc_graph = nullptr;
  const void* pc_in = nullptr;
  void* pc_out = nullptr;
  int pc_calls = 0;               // applications in the current solve
  bool pc_nograph = false;        // capture is not possible on the handle's stream
  double last_init_ms = 0.0;     // hierarchy construction (first solve only)
  double last_setup_ms = 0.0;    // phases of the last linear solve: diagonals + eigenvalue estimates,
  double last_rhs_ms = 0.0;      // right-hand side (+ inhomogeneous lift), CG iterations
  double last_iterate_ms = 0.0;
  // Newton blocks (NonlinearSolverParameters) and their block-vector work space
  int newton_max_iterations = 100;
  double newton_tolerance = 1e-10;
  double newton_step = 1.0;
  double* newton_update = nullptr;  // the change vector, kept between solves
  double* kv[8] = {};               // Krylov work vectors of the block length
  long long block_len = 0;
  int last_newton_iterations = 0;
  int last_newton_linear_iterations = 0;
  double last_newton_residual = 0.0;
  long long mesh_version = -1;      // mesh the work vectors were sized for (adaptive meshes)
};

struct BlockState {
  ppf_block_desc desc;
  BlockPlan plan[2];  // rhs, lhs
  LinearState lin;
};

}  // namespace ppf

struct ppf_handle_s {
  ppf_mesh_desc mesh;
  int dim = 2, k = 1, n = 2;
  int nc[3] = {1, 1, 1}, nn[3] = {1, 1, 1};
  double h[3] = {1, 1, 1};
  long long N = 0, ncells = 0;
  std::vector<ppf::FieldState> fields;
  std::vector<ppf::BlockState> blocks;
  const ppf::ModelOps* model = nullptr;
  ppf::ModelOps custom_ops{};              // operator compiled by the caller (ppf_create_custom)
  std::string custom_name;
  ppf_cell_launch_fn custom_launch = nullptr;
  std::vector<unsigned char> model_obj;
  std::vector<unsigned char> model_obj_f32;  // FP32 object (operator sets with an FP32 LHS)
  std::vector<double> constants;
  double* d_invm = nullptr;
  double* d_invm_sqrt = nullptr;
  std::vector<double> h_invm;
  int* d_err = nullptr;
  cudaStream_t stream = nullptr;      // stream all work is queued on
  cudaStream_t own_stream = nullptr;  // the handle's own stream
  cudaStream_t copy_stream = nullptr; // device-to-host copies of streamed outputs
  cudaEvent_t copy_ev = nullptr;
  bool copies_pending = false;
  cudaStream_t upload_stream = nullptr;  // host-to-device copies of staged uploads
  bool async_run = false;                // inside ppf_run_async: no host waits
  prismspf::SimulationTimer timer;
  double dt = 0.0;
  std::string err;
  bool use_graph = true;
  // NucleationRate blocks also run on increments divisible by this (nucleation_parameters.cc:110-113)
  unsigned int nucleation_period = 2147483647u;
  double* d_scratch_src = nullptr;  // ppf_apply host-path staging
  double* d_scratch_dst = nullptr;
  long long scratch_len = 0;
  ppf::AdjointState* adj = nullptr;  // adjoint / tangent-linear state (created on first use)
  ppf::AmrState* amr = nullptr;      // adaptive mesh (ppf_set_adaptivity), else null
  long long mesh_version = 0;
  long long graph_mesh_version = -1;  // mesh the increment graph was captured on
  long long state_version = 0;        // bumped when a staged upload swaps a state buffer in
  long long graph_state_version = -1; // state buffers the increment graph was captured on
  // CUDA graph of the explicit increment loop
  prismspf::SimulationTimer* d_timer = nullptr;
  cudaGraphExec_t run_graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  int graph_period = 0;
  long long graph_phase = 0;
  long long graph_launches = 0;
  long long rot_count = 0;
  bool capturing = false;
  // kernel timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  long long cell_launches = 0;
  long long all_launches = 0;
};

namespace ppf {

inline int fail(ppf_handle h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define PPF_CUDA(h, call)                                                                            \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return fail(h, PPF_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

unsigned grid_for(long long n);
int check_err(ppf_handle h);
double* state_ptr(ppf_handle h, int f, int age);
// records a kernel launch for the statistics; brackets cell launches with events when timing
int timed_cell_launch(ppf_handle h, int precision, int mode, const CellLaunch& L, const void* obj, size_t smem);
// plain_src: the LHS reads src without the homogeneous constraints (the inhomogeneous lift)
int launch_cell(ppf_handle h, int b, int which, const double* const* src, bool plain_src = false);
int linear_solve(ppf_handle h, int b);
int newton_solve(ppf_handle h, int b);
void free_linear(LinearState& L);
int explicit_solve_entry(ppf_handle h, int b);
struct AdjointState;
void free_adjoint(AdjointState* A);
// adaptive meshes (amr.cu)
int amr_launch_cell(ppf_handle h, int b, int which, const CellLaunch& L);
int amr_finalize_explicit(ppf_handle h, FieldState& F);
int amr_remesh_if_due(ppf_handle h);
unsigned amr_next_remesh(ppf_handle h, unsigned inc);
int amr_permute_io(ppf_handle h, int f, double* host, const double* dev_src, double* dev_dst, int ordering,
                   bool upload);
int amr_apply_constraints(ppf_handle h, FieldState& F, double* v);
// hanging entries of a host vector (ncomp components) from their masters
void amr_fill_hanging(ppf_handle h, int ncomp, double* v);
void free_amr(AmrState* A);

}  // namespace ppf
