/*
 * ppf_gb300.h — C ABI of the GB300 matrix-free operator-evaluation engine.
 *
 * Plain C: opaque handle, plain pointers and sizes, int status codes. No C++ or torch types
 * cross this boundary. Every entry point names the PRISMS-PF interface it replaces (paths
 * are inside prisms-center/phaseField).
 *
 * Vectors exchanged through this ABI are FP64. Their ordering is chosen per call:
 *   PPF_ORDER_LATTICE  lattice order: node (I,J,K) of the (k*Cx+1)x(k*Cy+1)x(k*Cz+1) node
 *                      lattice at index I + NX*(J + NY*K); vector fields component-major
 *                      (component c occupies [c*N, (c+1)*N)). Periodic images are kept,
 *                      as deal.II keeps periodic slave DoFs in the vector.
 *   PPF_ORDER_DEALII   the DoF numbering deal.II's DoFHandler::distribute_dofs produces for
 *                      the same mesh (cells in refinement order; per cell vertices, lines,
 *                      quads, hex interior; FESystem components per object).
 *   PPF_ORDER_NATIVE   the handle's own order: the lattice order on uniform meshes; on
 *                      adaptive meshes the DoFs in first-touch order over the active cells
 *                      (see ppf_set_adaptivity), vector fields component-major.
 *
 * Threading: a handle is not thread-safe; it owns one CUDA stream. Errors never throw:
 * every call returns PPF_OK or a PPF_ERR_* code, and ppf_last_error() gives the message.
 */
#ifndef PPF_GB300_H
#define PPF_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPF_MAX_FIELDS 8
#define PPF_MAX_BLOCKS 8
#define PPF_NAGE 6 /* dependency ages: current, old_1..old_4, src */

enum ppf_status {
  PPF_OK = 0,
  PPF_ERR_ARG = 1,          /* invalid argument */
  PPF_ERR_NAN = 2,          /* non-finite value after a solve (problem.cc:455-469 exit status 2) */
  PPF_ERR_CUDA = 3,         /* CUDA runtime error */
  PPF_ERR_NOCONV = 4,       /* linear solver did not converge (linear_solver.h:382-391) */
  PPF_ERR_DEPENDENCY = 5,   /* callback read an undeclared dependency (field_container.h:603-632) */
  PPF_ERR_UNSUPPORTED = 6,  /* configuration outside what this build implements */
  PPF_ERR_TIMEOUT = 7       /* a bounded device-side wait gave up */
};

enum ppf_ordering { PPF_ORDER_LATTICE = 0, PPF_ORDER_DEALII = 1, PPF_ORDER_NATIVE = 2 };

/* dependency flags (dependencies.h:134-213: values, grad(), hess()/lap()/hessdiag()) */
enum ppf_dep_flag { PPF_DEP_VALUE = 1, PPF_DEP_GRADIENT = 2, PPF_DEP_HESSIAN = 4 };

/* solve types / timings, same values as type_enums.h SolveType and solve_block.h SolveTiming */
enum ppf_solve_type { PPF_CONSTANT = 0, PPF_EXPLICIT = 1, PPF_LINEAR = 2, PPF_NEWTON = 3 };
enum ppf_solve_timing { PPF_PRIMARY = 0, PPF_SECONDARY = 1, PPF_POSTPROCESS = 2, PPF_NUCLEATION_RATE = 3 };

typedef struct ppf_handle_s* ppf_handle;

/* RectangularMesh + global refinement (spatial_discretization.cc:133-177,
 * triangulation_manager.cc:107-118): subdivided hyper-rectangle refined `global_refinement`
 * times; boundary ids x-=0, x+=1, y-=2, y+=3, z-=4, z+=5. */
typedef struct {
  int dim;                 /* 2 or 3 */
  int degree;              /* FE_Q degree 1..4 on Gauss-Lobatto points (system_wide.h:40-61) */
  int subdivisions[3];
  double lower[3];
  double size[3];
  int global_refinement;
  int periodic[3];         /* periodic directions (pairs 2d <-> 2d+1) */
} ppf_mesh_desc;

/* FieldAttributes + boundary conditions (field_attributes.h, constraint_parameters.cc:41-107).
 * dirichlet[c][b] != 0 makes component c Dirichlet on boundary id b with value
 * dirichlet_value[c][b] (the value set_dirichlet returns there; constant per face). */
typedef struct {
  int rank;                /* 0 scalar, 1 vector */
  int dirichlet[3][6];
  double dirichlet_value[3][6];
} ppf_field_desc;

/* SolveBlock (solve_block.h:56-127) with its dependency sets as flag tables:
 * dep_rhs[f][age] / dep_lhs[f][age] = OR of ppf_dep_flag, ages in the order
 * current, old_1, old_2, old_3, old_4, src (make_dependency_set result). */
typedef struct {
  int id;
  int solve_type;
  int solve_timing;
  int n_fields;
  int field_indices[PPF_MAX_FIELDS];
  unsigned char dep_rhs[PPF_MAX_FIELDS][PPF_NAGE];
  unsigned char dep_lhs[PPF_MAX_FIELDS][PPF_NAGE];
} ppf_block_desc;

/* Build the system once on the host and upload it: mesh, lattice/DoF maps, constraint maps,
 * inverse lumped mass, per-block cell tables (replaces Problem::init_system,
 * problem.cc:229-338). `model` names a compiled PDE operator set ("allen_cahn",
 * "cahn_hilliard", "eshelby", "coupled_acch"); `constants` are its Model constants in the
 * order that operator documents. */
int ppf_create(const ppf_mesh_desc* mesh, const ppf_field_desc* fields, int n_fields,
               const ppf_block_desc* blocks, int n_blocks, const char* model,
               const double* constants, int n_constants, double dt, ppf_handle* out);
void ppf_destroy(ppf_handle h);
const char* ppf_last_error(ppf_handle h);

/* A PDE operator compiled outside this library: the user's CustomPDE, instantiated by the
 * drop-in prismspf/core/problem.h in the user's own translation unit (the callbacks of
 * PDEOperatorBase::compute_rhs / compute_lhs, pde_operator_base.h:77-90). For every
 * cell-kernel launch the engine calls `launch` with its launch record (`cell_launch`, a
 * ppf::CellLaunch from prismspf/gpu/cell_kernel.cuh), the operator object bytes of the
 * requested precision (host memory; they travel as a kernel argument), the dynamic shared
 * memory size and the CUDA stream (a cudaStream_t). `launch` returns a cudaError_t value.
 * mode: 0 rhs, 1 lhs, 2 lhs diagonal probe; precision: 0 FP64, 1 FP32. */
typedef int (*ppf_cell_launch_fn)(int dim, int degree, int mode, int precision, const void* cell_launch,
                                  const void* object, size_t smem, void* stream);
typedef struct {
  const char* name;
  int has_lhs;                 /* compute_lhs is implemented (Linear blocks) */
  const void* object;          /* FP64 operator object bytes */
  size_t object_size;
  const void* object_f32;      /* FP32 operator object (mixed-precision smoothing) or NULL */
  size_t object_f32_size;
  ppf_cell_launch_fn launch;
  size_t cell_launch_size;     /* sizeof(ppf::CellLaunch) in the caller's build (layout check) */
} ppf_model_desc;

/* ppf_create for an operator compiled by the caller (Problem::Problem + init_system,
 * problem.cc:229-338, with the user's PDEOperatorBase). The object bytes are copied. */
int ppf_create_custom(const ppf_mesh_desc* mesh, const ppf_field_desc* fields, int n_fields,
                      const ppf_block_desc* blocks, int n_blocks, const ppf_model_desc* model, double dt,
                      ppf_handle* out);

/* Per-node Dirichlet values of field f (the values set_dirichlet returns at the boundary
 * support points, constraint_manager.cc:427-446): `values` is a lattice-order vector of the
 * field's length; the entries at Dirichlet-constrained positions are taken, the rest ignored.
 * Replaces the per-face constants of ppf_field_desc from this call on. */
int ppf_set_dirichlet_values(ppf_handle h, int field, const double* values);

/* Support points of cells [first_cell, first_cell + n_cells) in deal.II's active-cell order,
 * each cell's (degree+1)^dim points in FE_Q's local DoF order (vertices, lines, faces,
 * interior): the order VectorTools::interpolate visits them when it evaluates an initial
 * condition (solver_base.h:178-229). `out` receives lattice node indices, n_cells*(k+1)^dim. */
int ppf_dealii_cell_nodes(ppf_handle h, long long first_cell, long long n_cells, long long* out);

/* Streams field f to host memory after every increment: the device-to-host copy of an
 * explicitly solved field is queued on a copy stream as soon as its block's finalize kernel has
 * run, so it overlaps the blocks after it; fields no explicit block writes are copied at the end
 * of the increment. ppf_run / ppf_end_increment return after the copies completed (host then
 * holds the increment's solution, as ppf_download_solution would return it). host == NULL
 * stops streaming the field. Lattice (= native) order only; not on adaptive meshes; increments
 * with streamed outputs run as plain launches (no graph replay). Pinned host memory makes the
 * copies asynchronous. Engine-side addition: the reference writes outputs from host vectors. */
int ppf_set_output_stream(ppf_handle h, int f, double* host, int ordering);

/* The solution of field f as it stood at the end of the last increment's solves, before the
 * age rotation (what SolutionOutput writes, problem.cc:505-552). */
int ppf_download_solution(ppf_handle h, int field, double* host, int ordering);

/* sizes: lattice nodes per component, vector length of field f, cell count */
long long ppf_n_nodes(ppf_handle h);
long long ppf_field_length(ppf_handle h, int field);
long long ppf_n_cells(ppf_handle h);

/* deal.II DoF numbering of the scalar (rank 0) or vector (rank 1) handler as a map
 * dealii_index -> lattice index (dof_manager.cc:12-26). `out` has field_length entries. */
int ppf_dof_map(ppf_handle h, int rank, long long* out);

/* Constraint map of field f in lattice order: master index (>=0, itself when unconstrained)
 * or -1-j for the j-th Dirichlet row (constraint_manager.cc:258-304 after close()). */
int ppf_constraint_map(ppf_handle h, int field, int* out);

/* Inverse lumped mass of a scalar field in lattice order (invm_manager.h:121-239). */
int ppf_invm(ppf_handle h, double* out);

/* Field state I/O (GroupSolutionHandler current/old vectors). age 0 = current, 1..4 = old_k. */
int ppf_upload_state(ppf_handle h, int field, int age, const double* host, int ordering);

/* ppf_upload_state without the wait: the copy is queued on the handle's stream (so the next
 * solve reads it) and the call returns at once; `host` must stay unchanged until a call that
 * waits for the stream (ppf_run, ppf_solve_block, a download) returned. Lattice (= native)
 * order, uniform meshes. Engine-side addition for callers overlapping host work with copies. */
int ppf_upload_state_async(ppf_handle h, int f, int age, const double* host, int ordering);

/* Pipelined I/O for callers that feed every increment from host memory and read every result
 * back (no counterpart in the reference, whose vectors live in host memory; it replaces the
 * upload/solve/download sequence around Problem::solve_increment, problem.cc:416-557):
 *   ppf_upload_state_staged copies `host` (lattice order, pinned memory for overlap) into a
 *     device staging buffer of (field f, age) on the handle's upload stream right away, as soon
 *     as the previous staged upload of that (f, age) was consumed; the next run, before its
 *     first block, waits for it and swaps the staging buffer in as the state of that age (the
 *     state's former buffer becomes the staging buffer of the next upload; no device copy).
 *     `host` must stay unchanged until ppf_wait returned (or the run that consumes it ended).
 *     Device pointers of the state (ppf_state_device_ptr) change at that run.
 *   ppf_run_async queues the increments of ppf_run and returns without waiting: streamed
 *     outputs (ppf_set_output_stream) are copied out of a per-field staging copy, which the
 *     finalize kernel of an explicit block writes beside the state, so the next increment may
 *     start while the copy to the host is in flight; errors are reported by ppf_wait.
 *   ppf_wait waits for the queued runs, staged uploads and streamed-output copies, and returns
 *     their status (PPF_ERR_NAN, PPF_ERR_DEPENDENCY) like ppf_run. The host buffers of streamed
 *     outputs hold the last increment's results once it returned.
 * A caller that loops { stage inputs; ppf_run_async } overlaps the copies of increment k+1 with
 * the computation of increment k. Uniform meshes only. */
int ppf_upload_state_staged(ppf_handle h, int f, int age, const double* host);
int ppf_run_async(ppf_handle h, unsigned int n_increments, int output_every);
int ppf_wait(ppf_handle h);
int ppf_download_state(ppf_handle h, int field, int age, double* host, int ordering);

/* Apply the constraints of field f to its current vector (AffineConstraints::distribute,
 * group_solution_handler.cc:339-353). */
int ppf_apply_constraints(ppf_handle h, int field);

/* Increment loop of Problem::solve (problem.cc:341-557): runs increments from the current
 * one up to and including n_increments. Increment 0 applies the initial condition of
 * Primary blocks (uploaded beforehand) and solves Secondary blocks; PostProcess blocks run
 * on increments divisible by output_every (never when output_every <= 0). */
int ppf_run(ppf_handle h, unsigned int n_increments, int output_every);

/* The increment loop split open, for callers that act between blocks (the sharded driver
 * exchanges halo planes after every block): ppf_increment_block does block b's part of the
 * current increment exactly as ppf_run would (PostProcess blocks only when is_output,
 * NucleationRate blocks when is_output or on a nucleation-attempt increment; Primary blocks
 * keep the initial condition at increment 0; old ages start from the current vector at
 * increment 0); ppf_end_increment rotates the ages, advances the timer and reports a
 * non-finite result as PPF_ERR_NAN. */
int ppf_increment_block(ppf_handle h, int b, int is_output);

/* Nucleation-attempt period (the `nucleation period` entry of the `nucleation` subsection,
 * NucleationParameters::should_attempt_nucleation, src/user_inputs/nucleation_parameters.cc:
 * 110-113): NucleationRate blocks run on output increments and on increments divisible by the
 * period (problem.cc:436-443); the default is the reference's 2147483647, i.e. increment 0 and
 * output increments. Stochastic nucleation itself is not part of this engine. */
int ppf_set_nucleation_period(ppf_handle h, unsigned int period);
int ppf_end_increment(ppf_handle h);

/* One explicit solve of block index b (ExplicitSolver::solve_impl, explicit_solver.h:63-77). */
int ppf_solve_block(ppf_handle h, int b);

/* Operator apply of block b on host vectors (MFOperator::compute_operator / vmult,
 * mf_operator.cc:17-32, 304-310). which: 0 rhs (compute_rhs, plain reads), 1 lhs
 * (compute_lhs, src read with homogeneous constraints). src/dst: block fields concatenated
 * in block order, lattice order. scale: 0 none, 1 invM, 2 invM^(1/2). */
int ppf_apply(ppf_handle h, int b, int which, const double* src, double* dst, int scale);

/* Same on device pointers (no host copies); stream-ordered on the handle's stream. */
int ppf_apply_device(ppf_handle h, int b, int which, const double* d_src, double* d_dst, int scale);

/* SimulationTimer state (simulation_timer.h). */
int ppf_set_time(ppf_handle h, unsigned int increment, double time);
int ppf_get_time(ppf_handle h, unsigned int* increment, double* time);

/* LinearSolverParameters (src/user_inputs/solve_parameters.cc:10-187, same defaults): CG
 * preconditioned by nothing, Chebyshev (Jacobi-Chebyshev on the fine operator) or a GMG
 * V-cycle with Chebyshev smoothing and the smoother as coarse solve
 * (include/prismspf/solvers/linear_solver.h:47-213). The convergence test is
 * ||invM^1/2 (b - A x)|| < tolerance * normalisation (linear_solver.h:414-427).
 * mixed_precision = 1 runs the V-cycle's smoother, level operators and transfers in FP32
 * under the FP64 CG (GMG only); the coarse level, residuals and inner products stay FP64. */
typedef struct {
  int tolerance_type;      /* 0 AbsoluteResidual, 1 RMSEPerField, 2 IntegratedPerField, 3 RMSETotal, 4 IntegratedTotal */
  double tolerance;        /* default 1e-10 */
  int max_iterations;      /* default 100 */
  int preconditioner;      /* 0 None, 1 Chebyshev, 2 GMG */
  int mg_depth;            /* levels of the GMG hierarchy, finest included (default 1) */
  int smoother_degree;     /* Chebyshev polynomial degree (default 5) */
  double smoothing_range;  /* lambda_max / lambda_min of the Chebyshev interval (default 15) */
  int eig_cg_iterations;   /* CG steps of the largest-eigenvalue estimate (default 10) */
  int mixed_precision;     /* see above (default 0) */
  int solver_type;         /* 0 cg (SolverCG), 1 bicgstab (SolverBicgstab, for non-symmetric Newton
                              Jacobians); Linear blocks use cg */
} ppf_linear_params;

int ppf_default_linear_params(ppf_linear_params* p);
int ppf_set_linear_params(ppf_handle h, int block, const ppf_linear_params* p);

/* LinearSolver::solve_impl (linear_solver.h:305-345) for Linear block b: rhs from
 * compute_rhs, inhomogeneous Dirichlet values lifted with the plain-read LHS, CG from the
 * previous homogeneous solution, then constraints. Returns PPF_ERR_NOCONV when max_iterations
 * is reached (the solution is still written, as the reference logs and continues). */
int ppf_linear_solve(ppf_handle h, int b, int* iterations, double* residual);

/* Wall-clock phases of the last ppf_linear_solve of block b, in ms: construction of the
 * level hierarchy (first solve only, else 0), per-solve set-up (level diagonals and Chebyshev
 * eigenvalue estimates), right-hand side (compute_rhs and the inhomogeneous lift), and the CG
 * iterations. Outputs may be NULL. */
int ppf_linear_stats(ppf_handle h, int b, double* init_ms, double* setup_ms, double* rhs_ms, double* iterate_ms);

/* NonlinearSolverParameters of Newton block b (solve_parameters.cc:350-470): at most
 * max_iterations Newton steps (default 100), stop when the scaled residual norm is at most
 * tolerance * normalisation (default 1e-10), update u += step_length * change (default 1). */
int ppf_set_newton_params(ppf_handle h, int b, int max_iterations, double tolerance, double step_length);

/* NewtonSolver::solve_impl (newton_solver.h:73-156) for Newton block b over all its fields:
 * start from old_1, then repeat { apply constraints; R = S compute_rhs; stop if ||R|| is small
 * enough; solve S compute_lhs(change) = R with the block's linear parameters (cg or bicgstab,
 * no preconditioner, or Chebyshev for single-field blocks), warm-started from the previous
 * change; u += step_length * change }. Returns PPF_ERR_NOCONV after max_iterations steps (the
 * solution is kept, as the reference warns and continues). Outputs may be NULL. */
int ppf_newton_solve(ppf_handle h, int b, int* newton_iterations, int* linear_iterations, double* residual);

/* Matrix diagonal of the LHS of block b by unit probes, scaled by invM^1/2 when the
 * tolerance type is not AbsoluteResidual, zero entries set to one
 * (MFOperator::compute_diagonal, mf_operator.cc:82-101); lattice order, host output. */
int ppf_lhs_diagonal(ppf_handle h, int b, double* out);

/* ---- Adaptive meshes ----------------------------------------------------------------------
 * Mesh adaptivity of RefinementManager (src/core/refinement_manager.cc:42-439) with deal.II's
 * refinement smoothing, hanging-node constraints and solution transfer, for degrees 1 and 2.
 *
 * The mesh is a forest of quadtrees / octrees over the coarse subdivided rectangle. It starts
 * uniform at the global refinement (the initial condition is uploaded on that mesh, in lattice
 * order, as for a uniform handle). In the increment loop (problem.cc:488-499) the remeshing step
 * runs after the blocks of an increment: at increment 0 up to max - min passes (stopping when
 * the DoF count no longer changes), later one pass every remeshing_period increments. A pass
 * flags cells whose fields meet a criterion at any quadrature point for refinement (below
 * max_refinement) and the others for coarsening (above min_refinement), smooths the flags
 * (complete families only, 2:1 balance across faces, edges and vertices, refinement of
 * unrefined islands), refines/coarsens, renumbers, transfers every stored age (old nodes keep
 * their values, new nodes interpolate the old cell containing them), recomputes the inverse
 * lumped mass and distributes the new constraints.
 *
 * Numbering (PPF_ORDER_NATIVE): active cells in tree order (coarse cells lexicographic, children
 * depth-first in lexicographic child order), DoFs by first touch with lexicographic cell nodes.
 * Periodic images are one DoF. Hanging DoFs hold their interpolated values and have invM = 0.
 * ppf_n_nodes / ppf_n_cells / ppf_field_length report the current mesh. */
enum ppf_refine_flag { PPF_REFINE_VALUE = 1, PPF_REFINE_GRADIENT = 2 };

/* SpatialDiscretization (spatial_discretization.cc:372-523): levels count from the coarse mesh
 * (0); criteria as RefinementCriterion (grid_refiner_criterion.h): value in the open range
 * (value_lower, value_upper), gradient magnitude above gradient_lower; vector fields use their
 * l2 norms (and compare the gradient norm with the value range, as the reference does). */
typedef struct {
  int min_refinement;
  int max_refinement;
  int remeshing_period;    /* <= 0: only the passes at increment 0 */
  int n_criteria;
  int criterion_field[PPF_MAX_FIELDS];
  int criterion_flags[PPF_MAX_FIELDS];
  double value_lower[PPF_MAX_FIELDS];
  double value_upper[PPF_MAX_FIELDS];
  double gradient_lower[PPF_MAX_FIELDS];
} ppf_adaptivity;

/* Makes the handle's mesh adaptive; call right after ppf_create / ppf_create_custom (field
 * states are reset). Fails with PPF_ERR_UNSUPPORTED for degree > 2 or meshes too fine for the
 * position encoding. Linear and Newton blocks solve without a preconditioner on adaptive meshes
 * (the reference refuses multigrid with adaptivity); their warm starts restart from zero after
 * a remesh. */
int ppf_set_adaptivity(ppf_handle h, const ppf_adaptivity* a);

/* One remeshing pass now (RefinementManager::do_adaptive_refinement). */
int ppf_adapt(ppf_handle h);

/* The remeshing step of the current increment, as ppf_run does it after the blocks (for callers
 * of ppf_increment_block / ppf_end_increment). */
int ppf_remesh_if_due(ppf_handle h);

/* Counts mesh changes (0 before the first); callers that cache geometry compare it. */
long long ppf_mesh_version(ppf_handle h);

/* Wall-clock phases of the last remeshing pass in ms, 5 values: refinement criteria, flag
 * smoothing, the new mesh (refine/coarsen, numbering, hanging lines, transfer plan), transfer of
 * the stored vectors, set-up of the new mesh (device arrays, inverse mass, constraints). The
 * reference's "Refine Grid" timer section (refinement_manager.cc:53). */
int ppf_remesh_stats(ppf_handle h, double* phases_ms);

/* Active cells in tree order, 4 ints each: level, x, y, z (integer coordinates at that level;
 * the cell spans lower + size * [x, x+1] / (subdivisions * 2^level) per axis). Uniform handles
 * report their lattice cells at the global refinement. */
int ppf_cells(ppf_handle h, int* out);

/* DoF indices (PPF_ORDER_NATIVE) of every active cell's (degree+1)^dim nodes, lexicographic. */
int ppf_cell_dofs(ppf_handle h, int* out);

/* Coordinates of the DoFs (3 doubles each, PPF_ORDER_NATIVE). */
int ppf_node_points(ppf_handle h, double* out);

/* Closed hanging-node lines: count[p] entries for DoF p (0 when not hanging), then the
 * (master, weight) entries in ascending master order. Returns the total entry count (outputs
 * may be NULL to size them), or -1. */
long long ppf_hanging(ppf_handle h, int* count, int* master, double* weight);

/* Values of the non-uniform Dirichlet conditions of field f (set_dirichlet,
 * pde_operator_base.h:68-76) on adaptive meshes: the engine calls fn at every Dirichlet node of
 * every mesh it builds; without it the per-face constants of ppf_field_desc apply. */
typedef double (*ppf_dirichlet_fn)(void* user, int field, int component, int boundary_id, const double* point,
                                   double time);
int ppf_set_dirichlet_function(ppf_handle h, int field, ppf_dirichlet_fn fn, void* user);

/* ---- Ensembles --------------------------------------------------------------------------
 * Many independent explicit Allen-Cahn simulations (block 1 of
 * applications/allen_cahn/explicit/custom_pde.h:72-87) of uneven mesh size (2-D, natural
 * boundaries), degree 1 or 2 and parameters (m_well, kappa per instance), advanced together
 * by ONE kernel launch per time step; steps are replayed from a captured CUDA graph. No
 * counterpart in the reference, which runs one simulation per process. */
typedef struct ppf_ensemble_s* ppf_ensemble;

int ppf_ensemble_create(int n_instances, const ppf_mesh_desc* meshes, const double* m_well, const double* kappa,
                        double dt, ppf_ensemble* out);
void ppf_ensemble_destroy(ppf_ensemble e);
const char* ppf_ensemble_last_error(ppf_ensemble e);
long long ppf_ensemble_instance_length(ppf_ensemble e, int instance);
/* field of one instance in lattice order */
int ppf_ensemble_upload(ppf_ensemble e, int instance, const double* host);
int ppf_ensemble_download(ppf_ensemble e, int instance, double* host);
/* advance every instance by n_steps explicit steps (one launch per step) */
int ppf_ensemble_run(ppf_ensemble e, int n_steps, int use_graph);
/* times the candidate tile shapes and grid sizes on `steps` steps of this ensemble, keeps the
 * fastest and restores the state; outputs the best time per step and the choice */
int ppf_ensemble_autotune(ppf_ensemble e, int steps, double* best_ms, int* best_shape, int* best_grid);
int ppf_ensemble_synchronize(ppf_ensemble e);
int ppf_ensemble_set_stream(ppf_ensemble e, void* stream);

/* ---- Adjoint ------------------------------------------------------------------------------
 * Hand-written adjoint of the explicit step of a coupled_acch block (fields c, n; scalar,
 * unconstrained), used to calibrate Mc, Kn and the initial fields. No counterpart in the
 * reference. Vectors are the block fields concatenated (c then n), lattice order.
 *
 * ppf_adjoint_forward: runs n_steps explicit steps from the fields' current vectors (u_0),
 *   keeping n_snapshots checkpoint slots (u_0 included) placed by the binomial schedule; the
 *   fields' current vectors then hold u_K.
 * ppf_adjoint_backward: from dJ/du_K returns dJ/d(Mc, Kn) and dJ/du_0, recomputing the
 *   states it needs from the checkpoints; forward_steps reports the forward steps taken by the
 *   forward and backward calls together.
 * ppf_tangent_linear: forward-mode reference du_K = (dF^K)(du_0, dMc, dKn) along the same
 *   trajectory (state left unchanged).
 * ppf_checkpoint_schedule_cost: forward steps of the schedule for (n_steps, n_snapshots). */
int ppf_adjoint_forward(ppf_handle h, int block, int n_steps, int n_snapshots);
int ppf_adjoint_backward(ppf_handle h, const double* dJ_duK, double* dJ_dparams, double* dJ_du0,
                         long long* forward_steps);
int ppf_tangent_linear(ppf_handle h, int block, int n_steps, const double* du0, const double* dparams,
                       double* duK);
long long ppf_checkpoint_schedule_cost(int n_steps, int n_snapshots);

/* Replay the explicit increment loop of ppf_run from a CUDA graph (on by default): one graph
 * holds as many increments as the age-rotation period, each followed by a device-side timer
 * advance. Used from increment 2 on when every block is Explicit or Constant, no PostProcess
 * output is requested and kernel timing is off. */
int ppf_set_use_graph(ppf_handle h, int on);

/* Device pointer of a field state (for zero-copy callers), valid until the next rotation or
 * the next run that consumes a staged upload (ppf_upload_state_staged) of that field. */
int ppf_state_device_ptr(ppf_handle h, int field, int age, double** out);

/* Wait for all work queued on the handle's stream. */
int ppf_synchronize(ppf_handle h);

/* Run the handle's work on a caller-owned CUDA stream (a cudaStream_t passed as void*;
 * NULL restores the handle's own stream). No counterpart in the reference, which has no
 * device streams. */
int ppf_set_stream(ppf_handle h, void* stream);

/* Kernel timing for roofline measurements: while enabled, every cell-kernel launch is
 * bracketed by CUDA events on its stream. ppf_kernel_stats returns the summed event time
 * (ms) and launch count since the last reset, plus the launches of all engine kernels
 * (cell, finalize, vector kernels) issued since the last reset. Replaces the reference's
 * Timer::Scope sections (utilities/timer.cc:114-143) for the device path. */
int ppf_kernel_timing(ppf_handle h, int enable);
int ppf_kernel_stats(ppf_handle h, double* cell_ms, long long* cell_launches, long long* all_launches);
int ppf_kernel_stats_reset(ppf_handle h);

/* Contraction arithmetic of block b's operator (which: 0 rhs, 1 lhs) on a uniform mesh:
 * *mode = 0 FP64 contractions (degrees 3-4, or PPF_FP64_CONTRACTIONS=1), 1 exact fixed-point
 * derivatives with FP64 integration, 2 fixed-point derivatives and integration, 3 FP64
 * derivatives with fixed-point integration, 4 the lane kernel (cubic cells: derivatives,
 * integration and value terms all in fixed point, one cell per lane), -1 not chosen yet (the
 * first plain launch of an explicit right-hand side or of a left-hand side times 1, 2, 3 and,
 * on cubic cells, 4 and keeps the fastest; a linear or Newton right-hand side takes 4 on cubic
 * cells, else 1; PPF_CONTRACTION_MODE=1-4 fixes the mode, 4 falling back to 1 on other cells).
 * Engine-side only: the reference contracts in FP64 (fe_evaluation sum factorisation). */
int ppf_contraction_mode(ppf_handle h, int b, int which, int* mode);

/* Measures the current GPU's FP64 FMA throughput (TFLOP/s, FMA = 2 flops) with a
 * register-resident FMA loop; the denominator of FP64 roofline fractions. */
int ppf_device_fp64_peak(double* tflops);

/* One explicit Allen-Cahn step that allocates nothing. No counterpart in the reference: it
 * exists for callers that cannot allocate GPU memory at the point where they need a step
 * (for example code running inside a framework that owns every device allocation through
 * its own pool, or a fixed-memory loop where cudaMalloc/cudaFree are not allowed).
 *
 * Computes d_n_new = invM (.) A_rhs(d_n_old) for block 1 of the Allen-Cahn application
 * (constants m_well, kappa, time step dt) on `mesh` with natural boundary conditions, on the
 * given stream (a cudaStream_t as void*, NULL = default stream); no handle is needed.
 * d_n_old / d_n_new are caller-owned device vectors in lattice order.
 *
 * Limit: meshes of at most 1,048,576 lattice nodes (8 MiB accumulator); larger meshes, and
 * periodic meshes, return PPF_ERR_UNSUPPORTED with a message on stderr. The scratch is one
 * static device array that every GPU loading this library holds until exit. All calls share
 * it: each call clears what must start at zero, and calls whose GPU work overlaps race, so
 * issue them on one stream. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and the device's SM count; make that first call before any stream
 * capture. The step returns before its GPU work ends, so it cannot report a non-finite
 * result itself: ppf_allen_cahn_step_noalloc_status does. */
int ppf_allen_cahn_step_noalloc(const ppf_mesh_desc* mesh, double m_well, double kappa, double dt,
                                const double* d_n_old, double* d_n_new, void* stream);

/* Status of the last ppf_allen_cahn_step_noalloc on the current device (no counterpart in the
 * reference; the companion of the allocation-free step, and like it allocates nothing): waits
 * for `stream` (the step's stream, NULL = default stream), reads the step's error word from the
 * static scratch array into a host int and returns PPF_ERR_NAN when the step produced a
 * non-finite value (the reference's NaN exit status, problem.cc:455-469), else PPF_OK. A later
 * step overwrites the word; call this before the next step is issued. */
int ppf_allen_cahn_step_noalloc_status(void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PPF_GB300_H */
