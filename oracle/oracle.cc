// ORACLE — test infrastructure only.
//
// CPU restatement (FP64, C++17, OpenMP) of the PRISMS-PF matrix-free operator-evaluation
// path and of the deal.II pieces it calls. Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load this library; the product path never
// does.
//
// Parity status: the reference (deal.II >= 9.6 + MPI + p4est) cannot be built here and its
// own tests hold no golden vectors for this path, so this restatement is "parity unpinned"
// against the reference binary. It is pinned instead by analytic known answers (constant
// fields, mass conservation, discrete-Laplacian eigenvectors, patch tests) in tests/.
//
// What it restates, with the reference file each part follows (paths inside
// prisms-center/phaseField):
//   * GL support points and GL quadrature with degree+1 points (collocation)
//       include/prismspf/core/system_wide.h:40-61
//   * subdivided hyper-rectangle + refine_global, boundary ids 0..2d-1
//       src/user_inputs/spatial_discretization.cc:133-161,
//       src/core/triangulation_manager.cc:107-118
//   * DoF numbering in deal.II distribute_dofs order (cells in refinement order, per cell:
//     vertices, lines, quads, hex interior; FESystem component-major per object)
//       src/core/dof_manager.cc:12-26
//   * periodic + Dirichlet AffineConstraints with chain closing
//       src/core/constraint_manager.cc:143-304, spatial_discretization.cc:95-120,165-177
//   * lumped inverse mass with generic (periodic-only) constraints
//       include/prismspf/core/invm_manager.h:121-239
//   * cell loop: read_dof_values(_plain) -> evaluate -> user callback per q ->
//     integrate -> distribute_local_to_global with condensed constraints
//       src/solvers/mf_operator.cc:17-80, include/prismspf/core/field_container.h:794-882,
//       include/prismspf/core/field_container.h:1258-1314
//   * explicit solve  include/prismspf/solvers/explicit_solver.h:63-77
//   * time loop order, increment-0 handling, age rotation
//       src/core/problem.cc:341-557, include/prismspf/solvers/solver_base.h:103-131,
//       src/core/group_solution_handler.cc:356-403
//   * application callbacks: allen_cahn/explicit/custom_pde.h:72-101,
//     cahn_hilliard/explicit/custom_pde.h:91-131,
//     mechanics/eshelby_inclusion/custom_pde.h:55-92 (+ utilities/mechanics.h:39-109),
//     coupled_allen_cahn_cahn_hilliard/custom_pde.h:63-176
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------------------------------
// 1-D Gauss-Lobatto rule on [0,1] and the Lagrange derivative matrix at its points.
// system_wide.h:40-61 uses FE_Q(QGaussLobatto<1>(degree+1)) and QGaussLobatto(degree+1).
// ---------------------------------------------------------------------------------------
struct GL {
  int n = 0;
  double x[8] = {};
  double w[8] = {};
  double D[8][8] = {};  // D[q][j] = d/dx L_j (x_q) on [0,1]
};

static double legendre(int n, double x, double* dp) {
  double p0 = 1.0, p1 = x;
  if (n == 0) { if (dp) *dp = 0; return 1.0; }
  for (int k = 2; k <= n; ++k) {
    double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1; p1 = p2;
  }
  if (dp) *dp = n * (x * p1 - p0) / (x * x - 1.0);
  return p1;
}

static GL make_gl(int n) {
  GL g; g.n = n;
  const int N = n - 1;  // Legendre degree
  std::vector<double> t(n);
  t[0] = -1.0; t[n - 1] = 1.0;
  // interior points: roots of P'_N, Newton from Chebyshev-Gauss-Lobatto guesses
  for (int i = 1; i < n - 1; ++i) {
    double x = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100; ++it) {
      // f = P'_N(x), f' = P''_N(x) from the Legendre ODE
      double dp; double p = legendre(N, x, &dp);
      double d2p = (2.0 * x * dp - N * (N + 1.0) * p) / (1.0 - x * x);
      double dx = dp / d2p;
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    t[i] = x;
  }
  std::sort(t.begin(), t.end());
  for (int i = 0; i < n; ++i) {
    double p = legendre(N, t[i], nullptr);
    double w = 2.0 / (N * (N + 1.0) * p * p);
    g.x[i] = 0.5 * (t[i] + 1.0);
    g.w[i] = 0.5 * w;
  }
  // symmetrise the nodes exactly
  for (int i = 0; i < n / 2; ++i) {
    double a = 0.5 * (g.x[i] + (1.0 - g.x[n - 1 - i]));
    g.x[i] = a; g.x[n - 1 - i] = 1.0 - a;
    double w = 0.5 * (g.w[i] + g.w[n - 1 - i]);
    g.w[i] = w; g.w[n - 1 - i] = w;
  }
  if (n % 2 == 1) g.x[n / 2] = 0.5;
  // barycentric derivative matrix
  double bw[8];
  for (int j = 0; j < n; ++j) {
    double p = 1.0;
    for (int k = 0; k < n; ++k) if (k != j) p *= (g.x[j] - g.x[k]);
    bw[j] = 1.0 / p;
  }
  for (int q = 0; q < n; ++q) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == q) continue;
      g.D[q][j] = (bw[j] / bw[q]) / (g.x[q] - g.x[j]);
      diag -= g.D[q][j];
    }
    g.D[q][q] = diag;
  }
  return g;
}

// ---------------------------------------------------------------------------------------
// AffineConstraints restatement: a constrained dof i has entries (j, w) and inhomogeneity.
// close() substitutes constrained masters until every master is unconstrained.
// ---------------------------------------------------------------------------------------
struct Constraints {
  std::vector<char> constrained;
  std::vector<std::vector<std::pair<long, double>>> entries;
  std::vector<double> inhom;
  void reinit(long n) { constrained.assign(n, 0); entries.assign(n, {}); inhom.assign(n, 0.0); }
  bool is_constrained(long i) const { return constrained[i] != 0; }
  void add_line(long i) { constrained[i] = 1; entries[i].clear(); inhom[i] = 0.0; }
  void close() {
    const long n = (long)constrained.size();
    for (int pass = 0; pass < 16; ++pass) {
      bool changed = false;
      for (long i = 0; i < n; ++i) {
        if (!constrained[i]) continue;
        std::vector<std::pair<long, double>> out;
        double inh = inhom[i];
        bool any = false;
        for (auto& e : entries[i]) {
          if (constrained[e.first]) {
            any = true;
            inh += e.second * inhom[e.first];
            for (auto& f : entries[e.first]) out.push_back({f.first, e.second * f.second});
          } else {
            out.push_back(e);
          }
        }
        if (any) {
          std::sort(out.begin(), out.end());
          std::vector<std::pair<long, double>> merged;
          for (auto& e : out) {
            if (!merged.empty() && merged.back().first == e.first) merged.back().second += e.second;
            else merged.push_back(e);
          }
          entries[i] = merged; inhom[i] = inh; changed = true;
        }
      }
      if (!changed) break;
    }
  }
};

// ---------------------------------------------------------------------------------------
// Mesh + DoF handlers
// ---------------------------------------------------------------------------------------
struct DofHandler {
  int ncomp = 1;
  long ndofs = 0;
  std::vector<long> cell_dofs;            // [cell][comp][local lexicographic node]
  std::vector<std::array<int, 4>> lattice;  // per dof: global lattice I,J,K and component
};

struct Mesh {
  int dim = 2, k = 1, n = 2, nloc = 4;  // nloc = n^dim
  int nc[3] = {1, 1, 1};
  double lo[3] = {0, 0, 0}, len[3] = {1, 1, 1}, h[3] = {1, 1, 1};
  int periodic[3] = {0, 0, 0};
  long ncells = 0;
  std::vector<std::array<int, 3>> cells;  // cell integer coordinates, deal.II order
  GL gl;
  DofHandler dh[2];  // [0] scalar FE_Q, [1] FESystem(FE_Q, dim)
  int nnode[3] = {1, 1, 1};
  // adaptive meshes: `cells` holds coordinates at each cell's own level `lev`; node
  // positions are integers in units of the node spacing at level `maxlev`
  bool adaptive = false;
  std::vector<int> lev;
  int sub[3] = {1, 1, 1};
  int maxlev = 0;
  long E[3] = {1, 1, 1};                  // extent in position units
  std::vector<std::array<long, 3>> pos;   // node position of every scalar DoF
};

// cell extent (per-cell on adaptive meshes; the same expression len / (sub * 2^level) as the
// uniform mesh's h, so a uniform adaptive mesh has bit-identical geometry)
static inline void cell_h(const Mesh& m, long c, double* h) {
  for (int d = 0; d < 3; ++d) {
    if (!m.adaptive || d >= m.dim) h[d] = m.h[d];
    else h[d] = m.len[d] / (int)((long)m.sub[d] << m.lev[c]);
  }
}

// refine_global: children of a cell ordered lexicographically (x fastest), recursively.
static void build_cells(Mesh& m, const int* subdiv, int refine) {
  const int dim = m.dim;
  const int f = 1 << refine;
  for (int d = 0; d < 3; ++d) m.nc[d] = d < dim ? subdiv[d] * f : 1;
  m.cells.clear();
  const int nchild = 1 << dim;
  // coarse cells lexicographic (subdivided_hyper_rectangle), then recursive children
  for (int cz = 0; cz < (dim == 3 ? subdiv[2] : 1); ++cz)
    for (int cy = 0; cy < subdiv[1]; ++cy)
      for (int cx = 0; cx < subdiv[0]; ++cx) {
        std::vector<std::array<int, 3>> cur{{cx, cy, cz}};
        for (int r = 0; r < refine; ++r) {
          std::vector<std::array<int, 3>> nxt;
          nxt.reserve(cur.size() * nchild);
          for (auto& c : cur)
            for (int ch = 0; ch < nchild; ++ch)
              nxt.push_back({2 * c[0] + (ch & 1), 2 * c[1] + ((ch >> 1) & 1),
                             dim == 3 ? 2 * c[2] + ((ch >> 2) & 1) : 0});
          cur.swap(nxt);
        }
        for (auto& c : cur) m.cells.push_back(c);
      }
  m.ncells = (long)m.cells.size();
}

// The cell-local lattice offsets of the dofs on each geometric object, in deal.II
// distribute_dofs_on_cell order: vertices (v = x + 2y + 4z), lines, quads, hex interior.
// Line numbering (GeometryInfo): 2D: 0:x=0, 1:x=1, 2:y=0, 3:y=1. 3D: lines 0-3 on z=0 as in
// 2D, 4-7 on z=1, 8-11 along z at (x,y)=(0,0),(1,0),(0,1),(1,1). Dofs inside a line run
// from its lower to its upper vertex; face-interior dofs are lexicographic in the face's
// two tangential directions (lower axis fastest). Only degree >= 3 depends on these two
// within-object orders.
struct LocalObject { std::vector<std::array<int, 3>> nodes; };

static std::vector<LocalObject> local_objects(int dim, int k) {
  std::vector<LocalObject> objs;
  auto vtx = [&](int v) { return std::array<int, 3>{(v & 1) * k, ((v >> 1) & 1) * k, dim == 3 ? ((v >> 2) & 1) * k : 0}; };
  const int nv = 1 << dim;
  for (int v = 0; v < nv; ++v) objs.push_back({{vtx(v)}});
  // lines: (fixed coords, running axis)
  struct L { int axis; int a, b; };  // running axis, fixed values of the other two axes (in units of k)
  std::vector<std::array<int, 4>> lines;  // {axis, fx, fy, fz} fixed positions (0/1) for non-running axes
  if (dim == 2) {
    lines = {{1, 0, 0, 0}, {1, 1, 0, 0}, {0, 0, 0, 0}, {0, 0, 1, 0}};
  } else {
    lines = {{1, 0, 0, 0}, {1, 1, 0, 0}, {0, 0, 0, 0}, {0, 0, 1, 0},
             {1, 0, 0, 1}, {1, 1, 0, 1}, {0, 0, 0, 1}, {0, 0, 1, 1},
             {2, 0, 0, 0}, {2, 1, 0, 0}, {2, 0, 1, 0}, {2, 1, 1, 0}};
  }
  for (auto& l : lines) {
    LocalObject o;
    for (int t = 1; t < k; ++t) {
      std::array<int, 3> p{l[1] * k, l[2] * k, l[3] * k};
      p[l[0]] = t;
      o.nodes.push_back(p);
    }
    objs.push_back(o);
  }
  if (dim == 2) {
    LocalObject o;
    for (int b = 1; b < k; ++b)
      for (int a = 1; a < k; ++a) o.nodes.push_back({a, b, 0});
    objs.push_back(o);
  } else {
    for (int f = 0; f < 6; ++f) {
      const int nax = f / 2, side = (f % 2) * k;
      int t0 = nax == 0 ? 1 : 0;
      int t1 = nax == 2 ? 1 : 2;
      LocalObject o;
      for (int b = 1; b < k; ++b)
        for (int a = 1; a < k; ++a) {
          std::array<int, 3> p{0, 0, 0};
          p[nax] = side; p[t0] = a; p[t1] = b;
          o.nodes.push_back(p);
        }
      objs.push_back(o);
    }
    LocalObject o;
    for (int c = 1; c < k; ++c)
      for (int b = 1; b < k; ++b)
        for (int a = 1; a < k; ++a) o.nodes.push_back({a, b, c});
    objs.push_back(o);
  }
  return objs;
}

static void distribute_dofs(Mesh& m, int which) {
  DofHandler& d = m.dh[which];
  const int dim = m.dim, k = m.k, n = m.n;
  d.ncomp = which == 0 ? 1 : dim;
  const int nc = d.ncomp;
  const long NX = m.nnode[0], NY = m.nnode[1], NZ = m.nnode[2];
  std::vector<long> node_first(NX * NY * NZ, -1);  // first dof index of a lattice node
  auto objs = local_objects(dim, k);
  d.cell_dofs.assign((size_t)m.ncells * nc * m.nloc, -1);
  d.lattice.clear();
  long next = 0;
  for (long c = 0; c < m.ncells; ++c) {
    const auto& cc = m.cells[c];
    for (auto& o : objs) {
      // an object is numbered at once for all its nodes and components (component-major)
      bool fresh = true;
      for (auto& p : o.nodes) {
        long I = (long)cc[0] * k + p[0], J = (long)cc[1] * k + p[1], K = dim == 3 ? (long)cc[2] * k + p[2] : 0;
        if (node_first[(K * NY + J) * NX + I] >= 0) { fresh = false; break; }
      }
      if (o.nodes.empty() || !fresh) continue;
      const long npts = (long)o.nodes.size();
      long base = next;
      for (long t = 0; t < npts; ++t) {
        auto& p = o.nodes[t];
        long I = (long)cc[0] * k + p[0], J = (long)cc[1] * k + p[1], K = dim == 3 ? (long)cc[2] * k + p[2] : 0;
        node_first[(K * NY + J) * NX + I] = base + t;  // component 0 dof of this node
      }
      for (int comp = 0; comp < nc; ++comp)
        for (long t = 0; t < npts; ++t) {
          auto& p = o.nodes[t];
          d.lattice.push_back({cc[0] * k + p[0], cc[1] * k + p[1], dim == 3 ? cc[2] * k + p[2] : 0, comp});
        }
      next += npts * nc;
    }
  }
  d.ndofs = next;
  // node -> dof of component comp: node_first + comp * npts(object). Recover via lattice.
  std::vector<long> comp_dof((size_t)NX * NY * NZ * nc, -1);
  for (long i = 0; i < d.ndofs; ++i) {
    auto& L = d.lattice[i];
    comp_dof[(((long)L[2] * NY + L[1]) * NX + L[0]) * nc + L[3]] = i;
  }
  for (long c = 0; c < m.ncells; ++c) {
    const auto& cc = m.cells[c];
    for (int comp = 0; comp < nc; ++comp)
      for (int l = 0; l < m.nloc; ++l) {
        int a = l % n, b = (l / n) % n, e = dim == 3 ? l / (n * n) : 0;
        long I = (long)cc[0] * k + a, J = (long)cc[1] * k + b, K = (long)cc[2] * k + e;
        if (dim == 2) K = 0;
        d.cell_dofs[((size_t)c * nc + comp) * m.nloc + l] = comp_dof[((K * NY + J) * NX + I) * nc + comp];
      }
  }
}

// ---------------------------------------------------------------------------------------
// Problem: fields, constraints, states, blocks, model callback.
// ---------------------------------------------------------------------------------------
enum { DEP_VALUE = 1, DEP_GRAD = 2, DEP_HESS = 4 };
enum { AGE_CURRENT = 0, AGE_OLD1 = 1, AGE_OLD2 = 2, AGE_OLD3 = 3, AGE_OLD4 = 4, AGE_SRC = 5 };
constexpr int NAGE = 6;

struct Field {
  int rank = 0;  // 0 scalar, 1 vector
  // dirichlet[comp][boundary_id] = {is_dirichlet, value}
  int dir_on[3][6] = {};
  double dir_val[3][6] = {};
  Constraints cons;
  std::vector<double> cur;
  std::vector<double> old[4];
  int n_old = 0;
};

struct Problem;

// LinearSolverParameters (src/user_inputs/solve_parameters.cc:10-187)
struct LinParams {
  int tol_type = 0;          // 0 AbsoluteResidual, 1 RMSEPerField, 2 IntegratedPerField, 3 RMSETotal, 4 IntegratedTotal
  double tol = 1e-10;
  int max_its = 100;
  int precond = 0;           // 0 None, 1 Chebyshev, 2 GMG
  int mg_depth = 1;
  int degree = 5;
  double range = 15.0;
  int eig_its = 10;
  int solver = 0;            // 0 cg (SolverCG), 1 bicgstab (SolverBicgstab)
};

// NonlinearSolverParameters (src/user_inputs/solve_parameters.cc:350-470)
struct NewtonParams {
  int max_its = 100;
  double tol = 1e-10;
  double step = 1.0;
};

struct OLevel {
  Problem* P = nullptr;      // problem at this refinement (the finest level is the problem itself)
  bool owned = false;
  std::vector<double> inv_diag, x, b, r, u, Ax, t;
  double lmax = 0, lmin = 0;
  bool eig_done = false;
  // prolongation to the next finer level as triplets (fine dof, coarse dof, weight)
  std::vector<long> pf, pc;
  std::vector<double> pw;
};

struct Block {
  int id = 0, solve_type = 1, timing = 0;
  std::vector<int> fields;
  std::vector<std::array<int, NAGE>> dep_rhs, dep_lhs;  // [field][age] flags
  // linear solves
  LinParams lin;
  bool lin_init = false;
  std::vector<double> x_hom;
  std::vector<OLevel> levels;
  int last_its = 0;
  double last_res = 0.0;
  // Newton solves
  NewtonParams newton;
  std::vector<double> newton_update;  // the "change" vector, kept between solves
  int last_newton_its = 0;
  int last_newton_lin_its = 0;
  double last_newton_res = 0.0;
};

struct Model;

struct Problem {
  Mesh m;
  std::vector<Field> fields;
  std::vector<Block> blocks;
  Constraints generic[2];
  std::vector<double> jxw[2], invm[2], invm_sqrt[2];
  double dt = 0.0, time = 0.0;
  unsigned increment = 0;
  // nucleation-attempt period (nucleation_parameters.cc:110-113, default 2147483647)
  unsigned nucleation_period = 2147483647u;
  int model = 0;
  std::vector<double> params;
  int nthreads = 0;
  std::string err;
  int subdiv[3] = {1, 1, 1};
  int refine = 0;
  // mesh adaptivity (SpatialDiscretization: min/max refinement, remeshing period, criteria)
  struct Criterion { int field, flags; double vlo, vhi, glo; };
  int min_level = 0, max_level = 0, period = 0;
  std::vector<Criterion> criteria;
  Constraints hanging;  // closed hanging-node lines of the scalar DoFs
  ~Problem();
};

// Per-q view handed to the model callbacks (restates FieldContainer getters/setters,
// field_container.h:1065-1314).
struct QData {
  int dim;
  // value/gradient per (field, age, comp)
  const double* val;   // [field][age][comp]
  const double* grad;  // [field][age][comp][dir]
  double* out_val;     // [field][comp]
  double* out_grad;    // [field][comp][dir]
  char* out_flags;     // [field] bit0 value submitted, bit1 gradient submitted
  int nf;
  double x[3];         // quadrature point location
  double vol;          // element volume
  double v(int f, int age, int comp = 0) const { return val[(f * NAGE + age) * 3 + comp]; }
  double g(int f, int age, int comp, int dir) const { return grad[((f * NAGE + age) * 3 + comp) * 3 + dir]; }
  void set_value(int f, int comp, double x_) { out_val[f * 3 + comp] = x_; out_flags[f] |= 1; }
  void set_grad(int f, int comp, int dir, double x_) { out_grad[(f * 3 + comp) * 3 + dir] = x_; out_flags[f] |= 2; }
};

typedef void (*Callback)(const Problem& P, QData& q, int block_id, bool lhs);

// ---------------------------------------------------------------------------------------
// Model callbacks (the reference applications' compute_rhs / compute_lhs).
// ---------------------------------------------------------------------------------------
// allen_cahn/explicit/custom_pde.h:72-101. params: m_well, kappa. fields n(0), mg_n(1), f_tot(2)
static void cb_allen_cahn(const Problem& P, QData& q, int block_id, bool) {
  const double m_well = P.params[0], kappa = P.params[1];
  const int dim = q.dim;
  if (block_id == 1) {
    double n = q.v(0, AGE_OLD1);
    double f_well = 4.0 * n * (n - 1.0) * (n - 0.5);
    q.set_value(0, 0, n - P.dt * m_well * f_well);
    for (int d = 0; d < dim; ++d) q.set_grad(0, 0, d, -P.dt * kappa * m_well * q.g(0, AGE_OLD1, 0, d));
  } else if (block_id == 2) {
    double n = q.v(0, AGE_CURRENT);
    double g2 = 0;
    for (int d = 0; d < dim; ++d) g2 += q.g(0, AGE_CURRENT, 0, d) * q.g(0, AGE_CURRENT, 0, d);
    double f_chem = n * n * n * n - 2.0 * n * n * n + n * n;
    double f_grad = 0.5 * kappa * g2;
    q.set_value(1, 0, std::sqrt(g2));
    q.set_value(2, 0, f_chem + f_grad);
  }
}

// cahn_hilliard/explicit/custom_pde.h:91-131. params: McV, KcV, WcV. fields c(0), mu(1), f_tot(2)
static void cb_cahn_hilliard(const Problem& P, QData& q, int block_id, bool) {
  const double McV = P.params[0], KcV = P.params[1], WcV = P.params[2];
  const int dim = q.dim;
  if (block_id == 0) {
    q.set_value(0, 0, q.v(0, AGE_OLD1));
    for (int d = 0; d < dim; ++d) q.set_grad(0, 0, d, -McV * P.dt * q.g(1, AGE_OLD1, 0, d));
  } else if (block_id == 1) {
    double c = q.v(0, AGE_CURRENT);
    q.set_value(1, 0, WcV * c * (c - 1.0) * (c - 0.5));
    for (int d = 0; d < dim; ++d) q.set_grad(1, 0, d, KcV * q.g(0, AGE_CURRENT, 0, d));
  } else if (block_id == 2) {
    double c = q.v(0, AGE_CURRENT);
    double g2 = 0;
    for (int d = 0; d < dim; ++d) g2 += q.g(0, AGE_CURRENT, 0, d) * q.g(0, AGE_CURRENT, 0, d);
    q.set_value(2, 0, c * c * c * c - 2.0 * c * c * c + c * c + 0.5 * KcV * g2);
  }
}

// allen_cahn/implicit/custom_pde.h:70-125 (Newton block 1, post-processing block 2).
// params: m_well, kappa. fields n(0), mg_n(1), f_tot(2)
static void cb_allen_cahn_implicit(const Problem& P, QData& q, int block_id, bool lhs) {
  const double m_well = P.params[0], kappa = P.params[1], dt = P.dt;
  const int dim = q.dim;
  if (block_id == 1 && !lhs) {
    const double n = q.v(0, AGE_CURRENT), n_old = q.v(0, AGE_OLD1);
    const double f_well = 4.0 * n * (n - 1.0) * (n - 0.5);
    q.set_value(0, 0, n_old - n - dt * m_well * f_well);
    for (int d = 0; d < dim; ++d) q.set_grad(0, 0, d, -dt * kappa * m_well * q.g(0, AGE_CURRENT, 0, d));
  } else if (block_id == 1 && lhs) {
    const double n = q.v(0, AGE_CURRENT), dn = q.v(0, AGE_SRC);
    const double df_well = 12.0 * n * (n - 1.0) + 2.0;
    q.set_value(0, 0, dn * (1.0 + dt * m_well * df_well));
    for (int d = 0; d < dim; ++d) q.set_grad(0, 0, d, dt * kappa * m_well * q.g(0, AGE_SRC, 0, d));
  } else if (block_id == 2 && !lhs) {
    const double n = q.v(0, AGE_CURRENT);
    double g2 = 0;
    for (int d = 0; d < dim; ++d) g2 += q.g(0, AGE_CURRENT, 0, d) * q.g(0, AGE_CURRENT, 0, d);
    q.set_value(1, 0, std::sqrt(g2));
    q.set_value(2, 0, n * n * n * n - 2.0 * n * n * n + n * n + 0.5 * kappa * g2);
  }
}

// cahn_hilliard/implicit/custom_pde.h:90-160 (Newton block 0 over c and mu, post-processing
// block 2). params: McV, KcV, WcV. fields c(0), mu(1), f_tot(2)
static void cb_cahn_hilliard_implicit(const Problem& P, QData& q, int block_id, bool lhs) {
  const double McV = P.params[0], KcV = P.params[1], WcV = P.params[2], dt = P.dt;
  const int dim = q.dim;
  if (block_id == 0 && !lhs) {
    const double c = q.v(0, AGE_CURRENT), mu = q.v(1, AGE_CURRENT), c_old = q.v(0, AGE_OLD1);
    q.set_value(0, 0, c_old - c);
    for (int d = 0; d < dim; ++d) q.set_grad(0, 0, d, -(dt * McV * q.g(1, AGE_CURRENT, 0, d)));
    q.set_value(1, 0, mu - WcV * c * (c - 1.0) * (c - 0.5));
    for (int d = 0; d < dim; ++d) q.set_grad(1, 0, d, -(KcV * q.g(0, AGE_CURRENT, 0, d)));
  } else if (block_id == 0 && lhs) {
    const double c = q.v(0, AGE_CURRENT), dc = q.v(0, AGE_SRC), dmu = q.v(1, AGE_SRC);
    q.set_value(0, 0, dc);
    for (int d = 0; d < dim; ++d) q.set_grad(0, 0, d, dt * McV * q.g(1, AGE_SRC, 0, d));
    const double j_mu_c = -WcV * (0.5 + 3.0 * (c * (c - 1.0))) * dc;
    q.set_value(1, 0, -j_mu_c - dmu);
    for (int d = 0; d < dim; ++d) q.set_grad(1, 0, d, KcV * q.g(0, AGE_SRC, 0, d));
  } else if (block_id == 2 && !lhs) {
    const double c = q.v(0, AGE_CURRENT);
    double g2 = 0;
    for (int d = 0; d < dim; ++d) g2 += q.g(0, AGE_CURRENT, 0, d) * q.g(0, AGE_CURRENT, 0, d);
    q.set_value(2, 0, c * c * c * c - 2.0 * c * c * c + c * c + 0.5 * KcV * g2);
  }
}

// Voigt stress (utilities/mechanics.h:39-109): sigma = C : eps with engineering shears.
static void voigt_stress(int dim, const double* C, const double eps[3][3], double sig[3][3]) {
  const int nv = dim == 3 ? 6 : (dim == 2 ? 3 : 1);
  double e[6] = {}, s[6] = {};
  if (dim == 3) {
    e[0] = eps[0][0]; e[1] = eps[1][1]; e[2] = eps[2][2];
    e[3] = eps[1][2] + eps[2][1]; e[4] = eps[0][2] + eps[2][0]; e[5] = eps[0][1] + eps[1][0];
  } else if (dim == 2) {
    e[0] = eps[0][0]; e[1] = eps[1][1]; e[2] = eps[0][1] + eps[1][0];
  } else {
    e[0] = eps[0][0];
  }
  for (int i = 0; i < nv; ++i) { double a = 0; for (int j = 0; j < nv; ++j) a += C[i * 6 + j] * e[j]; s[i] = a; }
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) sig[i][j] = 0;
  if (dim == 3) {
    sig[0][0] = s[0]; sig[1][1] = s[1]; sig[2][2] = s[2];
    sig[1][2] = sig[2][1] = s[3]; sig[0][2] = sig[2][0] = s[4]; sig[0][1] = sig[1][0] = s[5];
  } else if (dim == 2) {
    sig[0][0] = s[0]; sig[1][1] = s[1]; sig[0][1] = sig[1][0] = s[2];
  } else {
    sig[0][0] = C[0] * eps[0][0];
  }
}

// Eigenstrain field of seeded spherical inclusions: eps* = e0 * sum_i 0.5(1 - tanh((r_i - R_i)/w)),
// capped at e0. params layout: [0..35] C (6x6 Voigt), [36] e0, [37] width, [38] n_incl,
// then 4 doubles per inclusion (cx, cy, cz, R). With n_incl == 0 the reference's single
// centred-at-origin inclusion of eshelby_inclusion/custom_pde.h:60-77 is used.
static double eigenstrain(const Problem& P, const double* x, int dim) {
  const double* p = P.params.data();
  const double e0 = p[36], width = p[37];
  const int ni = (int)p[38];
  if (ni == 0) {
    double r = 0; for (int d = 0; d < dim; ++d) r += x[d] * x[d];
    r = std::sqrt(r);
    return 0.01 * (0.5 + 0.5 * std::tanh(10.0 * (r - 10.0)));
  }
  double s = 0;
  for (int i = 0; i < ni; ++i) {
    const double* c = p + 39 + 4 * i;
    double r = 0; for (int d = 0; d < dim; ++d) r += (x[d] - c[d]) * (x[d] - c[d]);
    r = std::sqrt(r);
    s += 0.5 * (1.0 - std::tanh((r - c[3]) / width));
  }
  return e0 * std::min(s, 1.0);
}

// mechanics/eshelby_inclusion/custom_pde.h:55-92: block 1, field u (vector).
static void cb_eshelby(const Problem& P, QData& q, int block_id, bool lhs) {
  if (block_id != 1) return;
  const int dim = q.dim;
  const double* C = P.params.data();
  double eps[3][3] = {}, sig[3][3];
  if (lhs) {
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) eps[i][j] = 0.5 * (q.g(0, AGE_SRC, i, j) + q.g(0, AGE_SRC, j, i));
    voigt_stress(dim, C, eps, sig);
    for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) q.set_grad(0, i, j, sig[i][j]);
  } else {
    double s = eigenstrain(P, q.x, dim);
    for (int i = 0; i < dim; ++i) eps[i][i] = s;
    voigt_stress(dim, C, eps, sig);
    for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) q.set_grad(0, i, j, -sig[i][j]);
  }
}

// coupled_allen_cahn_cahn_hilliard/custom_pde.h:63-176. params: Mc, Mn, Kn.
// fields c(0), n(1), f_tot(2), mag_grad_c(3)
static void cb_coupled(const Problem& P, QData& q, int block_id, bool) {
  const double Mc = P.params[0], Mn = P.params[1], Kn = P.params[2];
  const double dt = P.dt;
  const double a0 = -1.6704, a1 = -4.776, a2 = 5.1622, a3 = -2.7375, a4 = 1.3687;
  const double b0 = -1.5924, b1 = -5.9746, b2 = 5.0;
  const int dim = q.dim;
  if (block_id == 0) {
    const double c = q.v(0, AGE_OLD1), n = q.v(1, AGE_OLD1);
    const double c2 = c * c, c3 = c * c2, c4 = c2 * c2;
    const double n2 = n * n, n3 = n * n2, n4 = n2 * n2, n5 = n * n4;
    const double fa = a0 + a1 * c + a2 * c2 + a3 * c3 + a4 * c4;
    const double fa_c = a1 + 2 * a2 * c + 3 * a3 * c2 + 4 * a4 * c3;
    const double fa_cc = 2 * a2 + 6 * a3 * c + 12 * a4 * c2;
    const double fb = b0 + b1 * c + b2 * c2;
    const double fb_c = b1 + 2 * b2 * c;
    const double fb_cc = 2 * b2;
    const double h = 10.0 * n3 - 15.0 * n4 + 6.0 * n5;
    const double hn = 30.0 * n2 - 60.0 * n3 + 30.0 * n4;
    const double dndt_val = -Mn * (fb - fa) * hn;
    for (int d = 0; d < dim; ++d) {
      const double cx = q.g(0, AGE_OLD1, 0, d), nx = q.g(1, AGE_OLD1, 0, d);
      const double mu_grad = -(cx * ((1.0 - h) * fa_cc + h * fb_cc) + nx * ((fb_c - fa_c) * hn));
      const double dcdt_vec = Mc * -mu_grad;
      q.set_grad(0, 0, d, -dt * dcdt_vec);
      q.set_grad(1, 0, d, -dt * (Kn * Mn * nx));
    }
    q.set_value(0, 0, c);
    q.set_value(1, 0, n + dt * dndt_val);
  } else if (block_id == 1) {
    const double c = q.v(0, AGE_CURRENT), n = q.v(1, AGE_CURRENT);
    const double c2 = c * c, c3 = c * c2, c4 = c2 * c2;
    const double n2 = n * n, n3 = n * n2, n4 = n2 * n2, n5 = n * n4;
    const double fa = a0 + a1 * c + a2 * c2 + a3 * c3 + a4 * c4;
    const double fb = b0 + b1 * c + b2 * c2;
    const double h = 10.0 * n3 - 15.0 * n4 + 6.0 * n5;
    double nn = 0, cc = 0;
    for (int d = 0; d < dim; ++d) {
      nn += q.g(1, AGE_CURRENT, 0, d) * q.g(1, AGE_CURRENT, 0, d);
      cc += q.g(0, AGE_CURRENT, 0, d) * q.g(0, AGE_CURRENT, 0, d);
    }
    q.set_value(2, 0, (1.0 - h) * fa + h * fb + 0.5 * Kn * nn);
    q.set_value(3, 0, std::sqrt(cc));
  }
}

static Callback callback_for(int model) {
  switch (model) {
    case ORC_MODEL_ALLEN_CAHN: return cb_allen_cahn;
    case ORC_MODEL_CAHN_HILLIARD: return cb_cahn_hilliard;
    case ORC_MODEL_ESHELBY: return cb_eshelby;
    case ORC_MODEL_COUPLED_ACCH: return cb_coupled;
    case ORC_MODEL_ALLEN_CAHN_IMPLICIT: return cb_allen_cahn_implicit;
    case ORC_MODEL_CAHN_HILLIARD_IMPLICIT: return cb_cahn_hilliard_implicit;
    default: return nullptr;
  }
}

// ---------------------------------------------------------------------------------------
// Constraints construction.
// ---------------------------------------------------------------------------------------
static long lattice_dof(const Mesh& m, int which, const std::vector<long>& node2dof, long I, long J, long K, int comp) {
  const int nc = m.dh[which].ncomp;
  return node2dof[(((K * m.nnode[1] + J) * m.nnode[0]) + I) * nc + comp];
}

static std::vector<long> node_to_dof(const Mesh& m, int which) {
  const DofHandler& d = m.dh[which];
  std::vector<long> out((size_t)m.nnode[0] * m.nnode[1] * m.nnode[2] * d.ncomp, -1);
  for (long i = 0; i < d.ndofs; ++i) {
    auto& L = d.lattice[i];
    out[((((long)L[2] * m.nnode[1]) + L[1]) * m.nnode[0] + L[0]) * d.ncomp + L[3]] = i;
  }
  return out;
}

// make_periodicity_constraints restated: the dof on the face with boundary id 2d+1 is
// constrained to the matching dof on boundary id 2d, weight 1 (chains closed later).
static void make_periodic(const Mesh& m, int which, Constraints& C) {
  const DofHandler& d = m.dh[which];
  auto n2d = node_to_dof(m, which);
  for (long i = 0; i < d.ndofs; ++i) {
    auto& L = d.lattice[i];
    for (int dir = 0; dir < m.dim; ++dir) {
      if (!m.periodic[dir]) continue;
      if (L[dir] != m.nnode[dir] - 1) continue;
      long I = L[0], J = L[1], K = L[2];
      if (dir == 0) I = 0; else if (dir == 1) J = 0; else K = 0;
      long master = lattice_dof(m, which, n2d, I, J, K, L[3]);
      if (!C.is_constrained(i)) {
        C.add_line(i);
        C.entries[i].push_back({master, 1.0});
      } else {
        // a second periodic direction for an already-constrained dof: keep the first
        // line (deal.II resolves the corner through the chain of the other direction)
      }
      break;
    }
  }
}

static bool on_boundary(const Mesh& m, const std::array<int, 4>& L, int bid) {
  const int dir = bid / 2;
  if (dir >= m.dim) return false;
  return (bid % 2 == 0) ? L[dir] == 0 : L[dir] == m.nnode[dir] - 1;
}

static void make_field_constraints_adaptive(Problem& P, int f);

static void make_field_constraints(Problem& P, int f) {
  if (P.m.adaptive) {
    make_field_constraints_adaptive(P, f);
    return;
  }
  Field& F = P.fields[f];
  const int which = F.rank;
  const DofHandler& d = P.m.dh[which];
  F.cons.reinit(d.ndofs);
  make_periodic(P.m, which, F.cons);
  // interpolate_boundary_values: boundary ids in ascending order, dofs not yet constrained
  for (int comp = 0; comp < d.ncomp; ++comp)
    for (int bid = 0; bid < 2 * P.m.dim; ++bid) {
      if (!F.dir_on[comp][bid]) continue;
      for (long i = 0; i < d.ndofs; ++i) {
        auto& L = d.lattice[i];
        if (L[3] != comp || !on_boundary(P.m, L, bid)) continue;
        if (F.cons.is_constrained(i)) continue;
        F.cons.add_line(i);
        F.cons.inhom[i] = F.dir_val[comp][bid];
      }
    }
  F.cons.close();
}

// ---------------------------------------------------------------------------------------
// Cell loop (the MFOperator::compute_local_operator restatement).
// ---------------------------------------------------------------------------------------
struct DepSlot { int field, age, flags; const double* vec; const Constraints* cons; bool constrained_read; int ncomp; };

// dst[field] vectors are indexed by block position
static void cell_loop(Problem& P, const Block& B, bool lhs, const std::vector<const double*>& src,
                      std::vector<double*>& dst, const std::vector<const Constraints*>& dst_cons,
                      Callback cb, bool plain_src = false) {
  Mesh& m = P.m;
  const int dim = m.dim, n = m.n, nloc = m.nloc;
  const auto& deps = lhs ? B.dep_lhs : B.dep_rhs;
  const int nf = (int)P.fields.size();
  std::vector<DepSlot> slots;
  for (int f = 0; f < nf; ++f)
    for (int age = 0; age < NAGE; ++age) {
      int fl = deps[f][age];
      if (!fl) continue;
      Field& F = P.fields[f];
      const double* vec = nullptr;
      bool cread = false;
      if (age == AGE_CURRENT) vec = F.cur.data();
      else if (age == AGE_SRC) {
        int pos = -1;
        for (size_t b = 0; b < B.fields.size(); ++b) if (B.fields[b] == f) pos = (int)b;
        if (pos < 0 || !src[pos]) continue;
        vec = src[pos];
        // LHS reads src with homogeneous constraints (field_container.h:817-832) unless the
        // operator is set to read plain (linear_solver.h:322-324)
        cread = lhs && !plain_src;
      } else vec = F.old[age - 1].data();
      slots.push_back({f, age, fl, vec, &F.cons, cread, F.rank == 0 ? 1 : dim});
    }
  const GL& gl = m.gl;
  // colouring for thread safety of the scatter: cell parity per axis
  int ncol = 1 << dim;
  bool serial = false;
  for (int d = 0; d < dim; ++d) if (m.periodic[d] && (m.nc[d] % 2)) serial = true;
  if (m.adaptive) serial = true;  // cells of different levels share DoFs across parity colours
  std::vector<std::vector<long>> colours(ncol);
  for (long c = 0; c < m.ncells; ++c) {
    auto& cc = m.cells[c];
    int col = (cc[0] & 1) | ((cc[1] & 1) << 1) | (dim == 3 ? ((cc[2] & 1) << 2) : 0);
    colours[serial ? 0 : col].push_back(c);
  }
  const int nbf = (int)B.fields.size();
  for (int col = 0; col < ncol; ++col) {
    const auto& cl = colours[col];
    const long ncl = (long)cl.size();
#pragma omp parallel if (!serial) num_threads(P.nthreads > 0 ? P.nthreads : omp_get_max_threads())
    {
      std::vector<double> loc((size_t)slots.size() * 3 * nloc);
      std::vector<double> qval((size_t)nf * NAGE * 3, 0.0), qgrad((size_t)nf * NAGE * 9, 0.0);
      std::vector<double> ov((size_t)nloc * nf * 3), og((size_t)nloc * nf * 9);
      std::vector<char> oflag(nf);
      std::vector<double> vals((size_t)slots.size() * 3 * nloc), grads((size_t)slots.size() * 9 * nloc);
      std::vector<double> res((size_t)nloc * 3);
#pragma omp for schedule(static)
      for (long ci = 0; ci < ncl; ++ci) {
        const long c = cl[ci];
        const auto& cc = m.cells[c];
        double hc[3];
        cell_h(m, c, hc);
        const double detJ = hc[0] * hc[1] * (dim == 3 ? hc[2] : 1.0);
        // gather + evaluate each dependency
        for (size_t s = 0; s < slots.size(); ++s) {
          const DepSlot& S = slots[s];
          const DofHandler& dh = m.dh[S.ncomp == 1 ? 0 : 1];
          for (int comp = 0; comp < S.ncomp; ++comp)
            for (int l = 0; l < nloc; ++l) {
              long gdof = dh.cell_dofs[((size_t)c * S.ncomp + comp) * nloc + l];
              double v;
              if (S.constrained_read && S.cons->is_constrained(gdof)) {
                v = 0.0;
                for (auto& e : S.cons->entries[gdof]) v += e.second * S.vec[e.first];
              } else {
                v = S.vec[gdof];
              }
              loc[(s * 3 + comp) * nloc + l] = v;
            }
          for (int comp = 0; comp < S.ncomp; ++comp) {
            const double* u = &loc[(s * 3 + comp) * nloc];
            for (int l = 0; l < nloc; ++l) {
              vals[(s * 3 + comp) * nloc + l] = u[l];
              int a = l % n, b = (l / n) % n, e = l / (n * n);
              int idx[3] = {a, b, e};
              int stride[3] = {1, n, n * n};
              for (int d = 0; d < dim; ++d) {
                double acc = 0.0;
                int base = l - idx[d] * stride[d];
                for (int j = 0; j < n; ++j) acc += gl.D[idx[d]][j] * u[base + j * stride[d]];
                grads[((s * 3 + comp) * 3 + d) * nloc + l] = acc / hc[d];
              }
            }
          }
        }
        // quadrature loop with the user callback
        std::fill(ov.begin(), ov.end(), 0.0);
        std::fill(og.begin(), og.end(), 0.0);
        std::fill(oflag.begin(), oflag.end(), 0);
        for (int l = 0; l < nloc; ++l) {
          for (size_t s = 0; s < slots.size(); ++s) {
            const DepSlot& S = slots[s];
            for (int comp = 0; comp < S.ncomp; ++comp) {
              qval[(S.field * NAGE + S.age) * 3 + comp] = vals[(s * 3 + comp) * nloc + l];
              for (int d = 0; d < dim; ++d)
                qgrad[((S.field * NAGE + S.age) * 3 + comp) * 3 + d] = grads[((s * 3 + comp) * 3 + d) * nloc + l];
            }
          }
          QData q;
          q.dim = dim; q.val = qval.data(); q.grad = qgrad.data();
          q.out_val = &ov[(size_t)l * nf * 3]; q.out_grad = &og[(size_t)l * nf * 9];
          q.out_flags = oflag.data(); q.nf = nf;
          int a = l % n, b = (l / n) % n, e = l / (n * n);
          q.x[0] = m.lo[0] + (cc[0] + gl.x[a]) * hc[0];
          q.x[1] = m.lo[1] + (cc[1] + gl.x[b]) * hc[1];
          q.x[2] = dim == 3 ? m.lo[2] + (cc[2] + gl.x[e]) * hc[2] : 0.0;
          q.vol = detJ;
          cb(P, q, B.id, lhs);
        }
        // integrate + distribute for each block field
        for (int bf = 0; bf < nbf; ++bf) {
          const int f = B.fields[bf];
          const int ncomp = P.fields[f].rank == 0 ? 1 : dim;
          const DofHandler& dh = m.dh[ncomp == 1 ? 0 : 1];
          for (int comp = 0; comp < ncomp; ++comp) {
            for (int l = 0; l < nloc; ++l) {
              int a = l % n, b = (l / n) % n, e = l / (n * n);
              int idx[3] = {a, b, e};
              int stride[3] = {1, n, n * n};
              double wq = gl.w[a] * gl.w[b] * (dim == 3 ? gl.w[e] : 1.0);
              double r = 0.0;
              if (oflag[f] & 1) r += ov[((size_t)l * nf + f) * 3 + comp] * wq * detJ;
              if (oflag[f] & 2) {
                for (int d = 0; d < dim; ++d) {
                  int base = l - idx[d] * stride[d];
                  double acc = 0.0;
                  for (int qd = 0; qd < n; ++qd) {
                    int lq = base + qd * stride[d];
                    int aq = lq % n, bq = (lq / n) % n, eq = lq / (n * n);
                    double wqq = gl.w[aq] * gl.w[bq] * (dim == 3 ? gl.w[eq] : 1.0);
                    acc += og[(((size_t)lq * nf + f) * 3 + comp) * 3 + d] * gl.D[qd][idx[d]] * wqq;
                  }
                  r += acc * detJ / hc[d];
                }
              }
              res[comp * nloc + l] = r;
            }
          }
          // distribute_local_to_global with constraints condensed
          const Constraints* C = dst_cons[bf];
          double* out = dst[bf];
          for (int comp = 0; comp < ncomp; ++comp)
            for (int l = 0; l < nloc; ++l) {
              long gdof = dh.cell_dofs[((size_t)c * ncomp + comp) * nloc + l];
              double r = res[comp * nloc + l];
              if (C && C->is_constrained(gdof)) {
                for (auto& e2 : C->entries[gdof]) out[e2.first] += e2.second * r;
              } else {
                out[gdof] += r;
              }
            }
        }
      }
    }
  }
}

// Operator diagonal by per-cell unit probes (MFOperator::compute_local_field_diagonal,
// src/solvers/mf_operator.cc:147-218): for each cell and local node i, the src dof values are
// the identity at node i (every component of a vector field, as identity<Rank>() submits),
// the callback runs at every quadrature point, the integrated entry at node i is kept, and
// the cell diagonal is distributed with the field's constraints. Single-field LHS blocks.
static void diag_loop(Problem& P, const Block& B, std::vector<double>& diag) {
  Mesh& m = P.m;
  const int dim = m.dim, n = m.n, nloc = m.nloc;
  const int f0 = B.fields[0];
  Field& F0 = P.fields[f0];
  const int ncomp = F0.rank == 0 ? 1 : dim;
  const DofHandler& dh = m.dh[ncomp == 1 ? 0 : 1];
  const int nf = (int)P.fields.size();
  const GL& gl = m.gl;
  Callback cb = callback_for(P.model);
  diag.assign(dh.ndofs, 0.0);
  std::vector<double> qval((size_t)nf * NAGE * 3, 0.0), qgrad((size_t)nf * NAGE * 9, 0.0);
  std::vector<double> ov((size_t)nloc * nf * 3), og((size_t)nloc * nf * 9);
  std::vector<char> oflag(nf);
  std::vector<double> grads((size_t)3 * 3 * nloc), vals((size_t)3 * nloc), cdiag((size_t)3 * nloc);
  for (long c = 0; c < m.ncells; ++c) {
    const auto& cc = m.cells[c];
    double hc[3];
    cell_h(m, c, hc);
    const double detJ = hc[0] * hc[1] * (dim == 3 ? hc[2] : 1.0);
    for (int i = 0; i < nloc; ++i) {
      // probe: identity at node i for every component
      for (int comp = 0; comp < ncomp; ++comp)
        for (int l = 0; l < nloc; ++l) vals[comp * nloc + l] = (l == i) ? 1.0 : 0.0;
      for (int comp = 0; comp < ncomp; ++comp)
        for (int l = 0; l < nloc; ++l) {
          int a = l % n, b = (l / n) % n, e = l / (n * n);
          int idx[3] = {a, b, e};
          int stride[3] = {1, n, n * n};
          for (int d = 0; d < dim; ++d) {
            double acc = 0.0;
            int base = l - idx[d] * stride[d];
            for (int j = 0; j < n; ++j) acc += gl.D[idx[d]][j] * vals[comp * nloc + base + j * stride[d]];
            grads[(comp * 3 + d) * nloc + l] = acc / hc[d];
          }
        }
      std::fill(ov.begin(), ov.end(), 0.0);
      std::fill(og.begin(), og.end(), 0.0);
      std::fill(oflag.begin(), oflag.end(), 0);
      for (int l = 0; l < nloc; ++l) {
        for (int comp = 0; comp < ncomp; ++comp) {
          qval[(f0 * NAGE + AGE_SRC) * 3 + comp] = vals[comp * nloc + l];
          for (int d = 0; d < dim; ++d)
            qgrad[((f0 * NAGE + AGE_SRC) * 3 + comp) * 3 + d] = grads[(comp * 3 + d) * nloc + l];
        }
        QData q;
        q.dim = dim; q.val = qval.data(); q.grad = qgrad.data();
        q.out_val = &ov[(size_t)l * nf * 3]; q.out_grad = &og[(size_t)l * nf * 9];
        q.out_flags = oflag.data(); q.nf = nf;
        int a = l % n, b = (l / n) % n, e = l / (n * n);
        q.x[0] = m.lo[0] + (cc[0] + gl.x[a]) * hc[0];
        q.x[1] = m.lo[1] + (cc[1] + gl.x[b]) * hc[1];
        q.x[2] = dim == 3 ? m.lo[2] + (cc[2] + gl.x[e]) * hc[2] : 0.0;
        q.vol = detJ;
        cb(P, q, B.id, true);
      }
      // integrate and keep the entry at node i
      int a = i % n, b = (i / n) % n, e = i / (n * n);
      int idx[3] = {a, b, e};
      int stride[3] = {1, n, n * n};
      for (int comp = 0; comp < ncomp; ++comp) {
        double r = 0.0;
        double wq = gl.w[a] * gl.w[b] * (dim == 3 ? gl.w[e] : 1.0);
        if (oflag[f0] & 1) r += ov[((size_t)i * nf + f0) * 3 + comp] * wq * detJ;
        if (oflag[f0] & 2)
          for (int d = 0; d < dim; ++d) {
            int base = i - idx[d] * stride[d];
            double acc = 0.0;
            for (int qd = 0; qd < n; ++qd) {
              int lq = base + qd * stride[d];
              int aq = lq % n, bq = (lq / n) % n, eq = lq / (n * n);
              double wqq = gl.w[aq] * gl.w[bq] * (dim == 3 ? gl.w[eq] : 1.0);
              acc += og[(((size_t)lq * nf + f0) * 3 + comp) * 3 + d] * gl.D[qd][idx[d]] * wqq;
            }
            r += acc * detJ / hc[d];
          }
        cdiag[comp * nloc + i] = r;
      }
    }
    // distribute the cell diagonal with the field's constraints
    for (int comp = 0; comp < ncomp; ++comp)
      for (int l = 0; l < nloc; ++l) {
        long g = dh.cell_dofs[((size_t)c * ncomp + comp) * nloc + l];
        double r = cdiag[comp * nloc + l];
        if (F0.cons.is_constrained(g)) {
          for (auto& e2 : F0.cons.entries[g]) diag[e2.first] += e2.second * r;
        } else {
          diag[g] += r;
        }
      }
  }
}

static void compute_invm(Problem& P) {
  Mesh& m = P.m;
  for (int which = 0; which < 2; ++which) {
    if (which == 1 && m.dim == 1) { }
    DofHandler& d = m.dh[which];
    Constraints& C = P.generic[which];
    C.reinit(d.ndofs);
    if (!m.adaptive) {
      make_periodic(m, which, C);
    } else {
      // adaptive meshes merge periodic images; hanging nodes are condensed because deal.II's
      // MatrixFree resolves them from the mesh (its hanging-node masks) whatever the generic
      // constraints hold
      const long N = (long)m.pos.size();
      for (int comp = 0; comp < d.ncomp; ++comp)
        for (long p = 0; p < N; ++p) {
          if (!P.hanging.is_constrained(p)) continue;
          C.add_line(comp * N + p);
          for (auto& e : P.hanging.entries[p]) C.entries[comp * N + p].push_back({comp * N + e.first, e.second});
        }
    }
    C.close();
    P.jxw[which].assign(d.ndofs, 0.0);
    const int dim = m.dim, n = m.n, nloc = m.nloc;
    for (long c = 0; c < m.ncells; ++c) {
      double hc[3];
      cell_h(m, c, hc);
      const double detJ = hc[0] * hc[1] * (dim == 3 ? hc[2] : 1.0);
      for (int comp = 0; comp < d.ncomp; ++comp)
        for (int l = 0; l < nloc; ++l) {
          int a = l % n, b = (l / n) % n, e = l / (n * n);
          double r = m.gl.w[a] * m.gl.w[b] * (dim == 3 ? m.gl.w[e] : 1.0) * detJ;
          long g = d.cell_dofs[((size_t)c * d.ncomp + comp) * nloc + l];
          if (C.is_constrained(g)) { for (auto& e2 : C.entries[g]) P.jxw[which][e2.first] += e2.second * r; }
          else P.jxw[which][g] += r;
        }
    }
    P.invm[which].resize(d.ndofs);
    P.invm_sqrt[which].resize(d.ndofs);
    for (long i = 0; i < d.ndofs; ++i) {
      double s = P.jxw[which][i];
      P.invm[which][i] = s == 0.0 ? 0.0 : 1.0 / s;
      P.invm_sqrt[which][i] = std::sqrt(P.invm[which][i]);
    }
  }
}

// AffineConstraints::distribute: constrained entries set from their masters + inhomogeneity
static void distribute(const Constraints& C, double* v) {
  const long n = (long)C.constrained.size();
  for (long i = 0; i < n; ++i) {
    if (!C.constrained[i]) continue;
    double s = C.inhom[i];
    for (auto& e : C.entries[i]) s += e.second * v[e.first];
    v[i] = s;
  }
}

// ExplicitSolver::solve_impl: u = invM (.) A_rhs, then constraints.
static void explicit_solve(Problem& P, const Block& B) {
  std::vector<double*> dst;
  std::vector<const Constraints*> cons;
  std::vector<const double*> src(B.fields.size(), nullptr);
  for (int f : B.fields) {
    Field& F = P.fields[f];
    std::fill(F.cur.begin(), F.cur.end(), 0.0);
    dst.push_back(F.cur.data());
    cons.push_back(&F.cons);
  }
  cell_loop(P, B, false, src, dst, cons, callback_for(P.model));
  for (int f : B.fields) {
    Field& F = P.fields[f];
    const auto& im = P.invm[F.rank];
    for (size_t i = 0; i < F.cur.size(); ++i) F.cur[i] *= im[i];
    distribute(F.cons, F.cur.data());
  }
}

// ---------------------------------------------------------------------------------------
// Linear solves (LinearSolver + MGContext, include/prismspf/solvers/linear_solver.h:47-553)
// for single-field Linear blocks.
// ---------------------------------------------------------------------------------------
Problem* make_problem(int dim, int degree, const int* subdiv, const double* lower, const double* size, int refine,
                      const int* periodic);
void finalize_fields(Problem& P);

Problem::~Problem() {
  for (auto& B : blocks)
    for (auto& L : B.levels)
      if (L.owned) delete L.P;
}

static bool scaled(const LinParams& p) { return p.tol_type != 0; }

// dst = S A src (S = invM^1/2 unless AbsoluteResidual); constrained rows stay zero
static void lhs_op(Problem& P, const Block& B, const double* src, double* dst, bool plain) {
  Field& F = P.fields[B.fields[0]];
  const size_t nd = F.cur.size();
  std::fill(dst, dst + nd, 0.0);
  std::vector<const double*> s{src};
  std::vector<double*> d{dst};
  std::vector<const Constraints*> c{&F.cons};
  cell_loop(P, B, true, s, d, c, callback_for(P.model), plain);
  if (scaled(B.lin))
    for (size_t i = 0; i < nd; ++i) dst[i] *= P.invm_sqrt[F.rank][i];
}

static long lattice_index(const Problem& P, int rank, long dof) {
  const auto& L = P.m.dh[rank].lattice[dof];
  const long N = (long)P.m.nnode[0] * P.m.nnode[1] * P.m.nnode[2];
  return (long)L[3] * N + ((long)L[2] * P.m.nnode[1] + L[1]) * P.m.nnode[0] + L[0];
}

static double dotp(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

static void compute_inv_diag(Problem& P, const Block& B, std::vector<double>& inv) {
  std::vector<double> d;
  diag_loop(P, B, d);
  Field& F = P.fields[B.fields[0]];
  inv.resize(d.size());
  for (size_t i = 0; i < d.size(); ++i) {
    double v = scaled(B.lin) ? d[i] * P.invm_sqrt[F.rank][i] : d[i];
    if (v == 0.0) v = 1.0;  // set_zero_entries_to_one
    inv[i] = 1.0 / v;
  }
}

static double tridiag_max(const std::vector<double>& a, const std::vector<double>& b) {
  const int m = (int)a.size();
  if (!m) return 1.0;
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; ++i) {
    double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  auto below = [&](double x) {
    int cnt = 0;
    double q = a[0] - x;
    if (q < 0) cnt++;
    for (int i = 1; i < m; ++i) {
      double qq = q == 0.0 ? 1e-300 : q;
      q = a[i] - x - b[i - 1] * b[i - 1] / qq;
      if (q < 0) cnt++;
    }
    return cnt;
  };
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (below(mid) >= m) hi = mid; else lo = mid;
    if (hi - lo <= 1e-14 * std::max(1.0, std::fabs(hi))) break;
  }
  return hi;
}

// largest eigenvalue estimate of P A on a level: eig_its CG steps on A x = pattern, x0 = 0,
// pattern (lattice index mod 11) minus its mean over the unconstrained rows
static void estimate_eig(OLevel& L, const Block& B) {
  Problem& P = *L.P;
  Field& F = P.fields[B.fields[0]];
  const size_t n = F.cur.size();
  std::vector<double> b(n, 0.0), x(n, 0.0), r, z(n), p, q(n);
  double mean = 0.0;
  long nfree = 0;
  for (size_t i = 0; i < n; ++i)
    if (!F.cons.is_constrained(i)) { mean += double(lattice_index(P, F.rank, i) % 11); nfree++; }
  mean /= std::max(1L, nfree);
  for (size_t i = 0; i < n; ++i)
    b[i] = F.cons.is_constrained(i) ? 0.0 : double(lattice_index(P, F.rank, i) % 11) - mean;
  r = b;
  for (size_t i = 0; i < n; ++i) z[i] = L.inv_diag[i] * r[i];
  p = z;
  double rz = dotp(r, z), r0 = dotp(r, r);
  std::vector<double> al, be;
  for (int it = 0; it < B.lin.eig_its; ++it) {
    lhs_op(P, B, p.data(), q.data(), false);
    double pq = dotp(p, q);
    if (pq <= 0.0 || !std::isfinite(pq)) break;
    double alpha = rz / pq;
    for (size_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    al.push_back(alpha);
    if (std::sqrt(dotp(r, r)) < 1e-10 * std::sqrt(r0)) break;
    for (size_t i = 0; i < n; ++i) z[i] = L.inv_diag[i] * r[i];
    double rzn = dotp(r, z);
    double beta = rzn / rz;
    rz = rzn;
    be.push_back(beta);
    for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  const int m = (int)al.size();
  std::vector<double> a(m), o(m > 0 ? m - 1 : 0);
  for (int i = 0; i < m; ++i) {
    a[i] = 1.0 / al[i] + (i > 0 ? be[i - 1] / al[i - 1] : 0.0);
    if (i + 1 < m) o[i] = std::sqrt(std::max(0.0, be[i])) / al[i];
  }
  L.lmax = 1.2 * tridiag_max(a, o);
  L.lmin = L.lmax / B.lin.range;
  L.eig_done = true;
}

// Chebyshev smoother (first kind) on L.x with right-hand side L.b
static void chebyshev(OLevel& L, const Block& B, bool zero_start) {
  Problem& P = *L.P;
  const size_t n = L.b.size();
  const double theta = 0.5 * (L.lmax + L.lmin), delta = 0.5 * (L.lmax - L.lmin), sigma = theta / delta;
  if (zero_start) std::fill(L.x.begin(), L.x.end(), 0.0);
  std::fill(L.u.begin(), L.u.end(), 0.0);
  double rho_prev = 1.0 / sigma;
  for (int k = 0; k < B.lin.degree; ++k) {
    bool have_ax = !(zero_start && k == 0);
    if (have_ax) lhs_op(P, B, L.x.data(), L.Ax.data(), false);
    double c1, c2;
    if (k == 0) { c1 = 0.0; c2 = 1.0 / theta; }
    else {
      double rho = 1.0 / (2.0 * sigma - rho_prev);
      c1 = rho * rho_prev;
      c2 = 2.0 * rho / delta;
      rho_prev = rho;
    }
    for (size_t i = 0; i < n; ++i) {
      double r = have_ax ? L.b[i] - L.Ax[i] : L.b[i];
      L.u[i] = c1 * L.u[i] + c2 * L.inv_diag[i] * r;
      L.x[i] += L.u[i];
    }
  }
}

// prolongation weights from level c to level c+1 (GL nodal interpolation, tensor product)
static void build_prolongation(OLevel& cl, OLevel& fl, int f) {
  Problem& C = *cl.P;
  Problem& Fp = *fl.P;
  const int rank = Fp.fields[f].rank;
  const Mesh& mc = C.m;
  const Mesh& mf = Fp.m;
  const int dim = mf.dim, k = mf.k, n = mf.n;
  auto n2d = node_to_dof(mc, rank);
  const DofHandler& dhf = mf.dh[rank];
  cl.pf.clear(); cl.pc.clear(); cl.pw.clear();
  for (long i = 0; i < dhf.ndofs; ++i) {
    const auto& Lf = dhf.lattice[i];
    int cidx[3][8]; double cw[3][8]; int cnt[3] = {1, 1, 1};
    cidx[1][0] = cidx[2][0] = 0; cw[1][0] = cw[2][0] = 1.0;
    for (int d = 0; d < dim; ++d) {
      const int I = Lf[d];
      const int ncf = mf.nc[d];
      const int cf = std::min(I / k, ncf - 1);
      const double xf = mf.gl.x[I - k * cf];
      const int cc = cf / 2;
      const double xc = ((cf % 2) + xf) * 0.5;
      cnt[d] = 0;
      for (int j = 0; j < n; ++j) {
        double Lj = 1.0;
        for (int mm = 0; mm < n; ++mm) if (mm != j) Lj *= (xc - mf.gl.x[mm]) / (mf.gl.x[j] - mf.gl.x[mm]);
        if (std::fabs(Lj) > 1e-14) { cidx[d][cnt[d]] = k * cc + j; cw[d][cnt[d]] = Lj; cnt[d]++; }
      }
    }
    for (int a = 0; a < cnt[0]; ++a)
      for (int b = 0; b < cnt[1]; ++b)
        for (int c = 0; c < cnt[2]; ++c) {
          long I = cidx[0][a], J = dim > 1 ? cidx[1][b] : 0, K = dim > 2 ? cidx[2][c] : 0;
          long cd = lattice_dof(mc, rank, n2d, I, J, K, Lf[3]);
          cl.pf.push_back(i);
          cl.pc.push_back(cd);
          cl.pw.push_back(cw[0][a] * (dim > 1 ? cw[1][b] : 1.0) * (dim > 2 ? cw[2][c] : 1.0));
        }
  }
}

// homogeneous distribute: images take their master's value, Dirichlet rows zero
static void homogeneous_distribute(const Constraints& C, std::vector<double>& v) {
  for (size_t i = 0; i < v.size(); ++i) {
    if (!C.constrained[i]) continue;
    double s = 0.0;
    for (auto& e : C.entries[i]) s += e.second * v[e.first];
    v[i] = s;
  }
}

// condensation of a restricted vector: images add into masters, constrained rows zero
static void condense(const Constraints& C, std::vector<double>& v) {
  for (size_t i = 0; i < v.size(); ++i) {
    if (!C.constrained[i]) continue;
    for (auto& e : C.entries[i]) v[e.first] += e.second * v[i];
  }
  for (size_t i = 0; i < v.size(); ++i) if (C.constrained[i]) v[i] = 0.0;
}

static void vcycle(Block& Bfine, int l) {
  OLevel& L = Bfine.levels[l];
  Problem& P = *L.P;
  const Block& LB = *std::find_if(P.blocks.begin(), P.blocks.end(), [&](const Block& x) { return x.id == Bfine.id; });
  if (l == 0) { chebyshev(L, LB, true); return; }
  chebyshev(L, LB, true);
  lhs_op(P, LB, L.x.data(), L.r.data(), false);
  for (size_t i = 0; i < L.r.size(); ++i) L.r[i] = L.b[i] - L.r[i];
  OLevel& C = Bfine.levels[l - 1];
  std::fill(C.b.begin(), C.b.end(), 0.0);
  for (size_t q = 0; q < C.pf.size(); ++q) C.b[C.pc[q]] += C.pw[q] * L.r[C.pf[q]];
  condense(C.P->fields[LB.fields[0]].cons, C.b);
  vcycle(Bfine, l - 1);
  std::fill(L.t.begin(), L.t.end(), 0.0);
  for (size_t q = 0; q < C.pf.size(); ++q) L.t[C.pf[q]] += C.pw[q] * C.x[C.pc[q]];
  homogeneous_distribute(P.fields[LB.fields[0]].cons, L.t);
  for (size_t i = 0; i < L.x.size(); ++i) L.x[i] += L.t[i];
  chebyshev(L, LB, false);
}

static void init_linear(Problem& P, Block& B) {
  const int f = B.fields[0];
  const int R = P.refine;
  int depth = B.lin.precond == 2 ? std::max(1, B.lin.mg_depth) : 1;
  depth = std::min(depth, R + 1);
  B.levels.assign(depth, OLevel());
  for (int l = 0; l < depth; ++l) {
    OLevel& L = B.levels[l];
    if (l == depth - 1) {
      L.P = &P;
    } else {
      const int r = R - depth + 1 + l;
      double lo[3], sz[3];
      int per[3];
      for (int d = 0; d < 3; ++d) { lo[d] = P.m.lo[d]; sz[d] = P.m.len[d]; per[d] = P.m.periodic[d]; }
      Problem* C = make_problem(P.m.dim, P.m.k, P.subdiv, lo, sz, r, per);
      for (auto& F : P.fields) {
        Field G;
        G.rank = F.rank;
        std::memcpy(G.dir_on, F.dir_on, sizeof(G.dir_on));
        for (int c = 0; c < 3; ++c) for (int b = 0; b < 6; ++b) G.dir_val[c][b] = 0.0;  // homogeneous
        C->fields.push_back(G);
      }
      C->blocks = P.blocks;
      for (auto& Bc : C->blocks) { Bc.levels.clear(); Bc.lin_init = false; }
      C->model = P.model;
      C->params = P.params;
      C->dt = P.dt;
      C->nthreads = P.nthreads;
      finalize_fields(*C);
      L.P = C;
      L.owned = true;
    }
    const size_t n = L.P->fields[f].cur.size();
    for (auto* v : {&L.x, &L.b, &L.r, &L.u, &L.Ax, &L.t}) v->assign(n, 0.0);
  }
  for (int l = 0; l + 1 < depth; ++l) build_prolongation(B.levels[l], B.levels[l + 1], f);
  B.x_hom.assign(P.fields[f].cur.size(), 0.0);
  B.lin_init = true;
}

// LinearSolver::normalization_value (linear_solver.h:414-427)
static double normalization(const Problem& P, const LinParams& p, int n_fields = 1) {
  double v = 1.0;
  if (p.tol_type == 1 || p.tol_type == 3) {
    double vol = 1.0;
    for (int d = 0; d < P.m.dim; ++d) vol *= P.m.len[d];
    v *= std::sqrt(vol);
  }
  if (p.tol_type == 1 || p.tol_type == 2) v *= std::sqrt((double)n_fields);
  return v;
}

// LinearSolver::solve_impl (linear_solver.h:305-345)
static int linear_solve(Problem& P, Block& B) {
  if (!B.lin_init) init_linear(P, B);
  const int f = B.fields[0];
  Field& F = P.fields[f];
  const size_t n = F.cur.size();
  // level diagonals (recomputed every solve) and eigenvalue estimates (first use)
  if (B.lin.precond != 0)
    for (auto& L : B.levels) {
      const Block& LB = *std::find_if(L.P->blocks.begin(), L.P->blocks.end(), [&](const Block& x) { return x.id == B.id; });
      compute_inv_diag(*L.P, LB, L.inv_diag);
      if (!L.eig_done) {
        Block tmp = LB;
        tmp.lin = B.lin;
        estimate_eig(L, tmp);
      }
    }
  // rhs = S compute_rhs
  std::vector<double> rhs(n, 0.0), g(n, 0.0), Ag(n), r(n), z(n), p(n), q(n);
  {
    std::vector<const double*> s{nullptr};
    std::vector<double*> d{rhs.data()};
    std::vector<const Constraints*> c{&F.cons};
    cell_loop(P, B, false, s, d, c, callback_for(P.model));
    if (scaled(B.lin)) for (size_t i = 0; i < n; ++i) rhs[i] *= P.invm_sqrt[F.rank][i];
  }
  distribute(F.cons, g.data());  // inhomogeneous values
  lhs_op(P, B, g.data(), Ag.data(), true);
  for (size_t i = 0; i < n; ++i) rhs[i] -= Ag[i];
  // CG (deal.II SolverCG) from the previous homogeneous solution
  std::vector<double>& x = B.x_hom;
  const double tol = B.lin.tol * normalization(P, B.lin);
  auto precond = [&](const std::vector<double>& rr, std::vector<double>& zz) {
    if (B.lin.precond == 0) { zz = rr; return; }
    OLevel& Lf = B.levels.back();
    Lf.b = rr;
    if (B.lin.precond == 1) chebyshev(Lf, B, true);
    else vcycle(B, (int)B.levels.size() - 1);
    zz = Lf.x;
  };
  lhs_op(P, B, x.data(), q.data(), false);
  for (size_t i = 0; i < n; ++i) r[i] = rhs[i] - q[i];
  double res = std::sqrt(dotp(r, r));
  int it = 0;
  bool conv = res < tol;
  if (!conv) {
    precond(r, z);
    p = z;
    double rz = dotp(r, z);
    while (it < B.lin.max_its) {
      lhs_op(P, B, p.data(), q.data(), false);
      double alpha = rz / dotp(p, q);
      for (size_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
      ++it;
      res = std::sqrt(dotp(r, r));
      if (res < tol) { conv = true; break; }
      precond(r, z);
      double rzn = dotp(r, z);
      double beta = rzn / rz;
      rz = rzn;
      for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
  }
  B.last_its = it;
  B.last_res = res / normalization(P, B.lin);
  for (size_t i = 0; i < n; ++i) F.cur[i] = x[i] + g[i];
  distribute(F.cons, F.cur.data());
  return conv ? 0 : 4;
}

// ---------------------------------------------------------------------------------------
// Newton solves over all fields of a block (NewtonSolver::solve_impl, newton_solver.h:73-156,
// with LinearSolver::do_linear_solve, linear_solver.h:348-402). Block vectors concatenate the
// block's fields in block order.
// ---------------------------------------------------------------------------------------
static std::vector<size_t> block_offsets(const Problem& P, const Block& B) {
  std::vector<size_t> off{0};
  for (int f : B.fields) off.push_back(off.back() + P.fields[f].cur.size());
  return off;
}

// dst = S op(src) over the block fields; which 0: compute_rhs (src unused), 1: compute_lhs
static void block_op(Problem& P, const Block& B, int which, const double* src, double* dst) {
  const auto off = block_offsets(P, B);
  std::vector<const double*> s;
  std::vector<double*> d;
  std::vector<const Constraints*> c;
  for (size_t i = 0; i < B.fields.size(); ++i) {
    Field& F = P.fields[B.fields[i]];
    s.push_back(src ? src + off[i] : nullptr);
    std::fill(dst + off[i], dst + off[i + 1], 0.0);
    d.push_back(dst + off[i]);
    c.push_back(&F.cons);
  }
  cell_loop(P, B, which == 1, s, d, c, callback_for(P.model));
  if (scaled(B.lin))
    for (size_t i = 0; i < B.fields.size(); ++i) {
      Field& F = P.fields[B.fields[i]];
      for (size_t j = 0; j < off[i + 1] - off[i]; ++j) dst[off[i] + j] *= P.invm_sqrt[F.rank][j];
    }
}

// Krylov solve of S A x = b (SolverCG or SolverBicgstab) from the initial guess in x;
// preconditioner: identity, or for a single-field block the Chebyshev smoother of the fine
// level. Returns the number of iterations; *conv tells whether the tolerance was reached.
static int block_krylov(Problem& P, Block& B, const std::vector<double>& b, std::vector<double>& x, double tol,
                        bool* conv, double* final_res) {
  const size_t n = b.size();
  auto A = [&](const std::vector<double>& v, std::vector<double>& out) { block_op(P, B, 1, v.data(), out.data()); };
  auto M = [&](const std::vector<double>& rr, std::vector<double>& zz) {
    if (B.lin.precond == 0) { zz = rr; return; }
    OLevel& Lf = B.levels.back();
    Lf.b = rr;
    chebyshev(Lf, B, true);
    zz = Lf.x;
  };
  std::vector<double> r(n), q(n);
  A(x, q);
  for (size_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
  double res = std::sqrt(dotp(r, r));
  int it = 0;
  *conv = res < tol;
  if (!*conv && B.lin.solver == 0) {
    std::vector<double> z(n), p(n);
    M(r, z);
    p = z;
    double rz = dotp(r, z);
    while (it < B.lin.max_its) {
      A(p, q);
      const double alpha = rz / dotp(p, q);
      for (size_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
      ++it;
      res = std::sqrt(dotp(r, r));
      if (res < tol) { *conv = true; break; }
      M(r, z);
      const double rzn = dotp(r, z);
      const double beta = rzn / rz;
      rz = rzn;
      for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
  } else if (!*conv) {
    // BiCGStab (van der Vorst), right-preconditioned, with the half-step convergence check
    std::vector<double> rbar = r, p(n, 0.0), v(n, 0.0), y(n), s(n), zz(n), t(n);
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int restarts = 0;
    // a breakdown (rho or omega zero, or |alpha| > 1e10) restarts from the current iterate with
    // the exact residual, as deal.II's SolverBicgstab (solver_bicgstab.h, iterate/solve) does;
    // at most 10 restarts
    auto restart = [&]() -> bool {
      A(x, q);
      for (size_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
      rbar = r;
      std::fill(p.begin(), p.end(), 0.0);
      std::fill(v.begin(), v.end(), 0.0);
      rho = alpha = omega = 1.0;
      res = std::sqrt(dotp(r, r));  // a breakdown right at convergence ends the solve
      return res < tol;
    };
    while (it < B.lin.max_its) {
      const double rho_new = dotp(rbar, r);
      if (rho_new == 0.0 || omega == 0.0) {  // breakdown
        if (++restarts > 10) break;
        if (restart()) { *conv = true; break; }
        continue;
      }
      const double beta = (rho_new / rho) * (alpha / omega);
      rho = rho_new;
      for (size_t i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
      M(p, y);
      A(y, v);
      const double sigma = dotp(rbar, v);
      if (sigma == 0.0 || !(std::fabs(rho / sigma) <= 1e10)) {  // breakdown
        if (++restarts > 10) break;
        if (restart()) { *conv = true; break; }
        continue;
      }
      alpha = rho / sigma;
      for (size_t i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
      ++it;
      const double sres = std::sqrt(dotp(s, s));
      if (sres < tol) {
        for (size_t i = 0; i < n; ++i) x[i] += alpha * y[i];
        res = sres;
        *conv = true;
        break;
      }
      M(s, zz);
      A(zz, t);
      const double tt = dotp(t, t);
      omega = tt > 0.0 ? dotp(t, s) / tt : 0.0;
      for (size_t i = 0; i < n; ++i) {
        x[i] += alpha * y[i] + omega * zz[i];
        r[i] = s[i] - omega * t[i];
      }
      res = std::sqrt(dotp(r, r));
      if (res < tol) { *conv = true; break; }
    }
  }
  *final_res = res;
  return it;
}

static int newton_solve(Problem& P, Block& B) {
  const int nbf = (int)B.fields.size();
  if (B.lin.precond == 2) return 6;               // GMG levels would need the current solution
  if (B.lin.precond == 1 && nbf != 1) return 6;   // Chebyshev: single-field blocks
  if (B.lin.precond == 1 && !B.lin_init) init_linear(P, B);
  const auto off = block_offsets(P, B);
  const size_t n = off.back();
  if (B.newton_update.size() != n) B.newton_update.assign(n, 0.0);
  // start from the previous solution (old_1 where the field keeps one)
  for (int f : B.fields) {
    Field& F = P.fields[f];
    if (F.n_old > 0) F.cur = F.old[0];
  }
  const double norm = normalization(P, B.lin, nbf);
  const double tol = B.newton.tol * norm;
  const double lin_tol = B.lin.tol * norm;
  std::vector<double> R(n);
  double l2 = -1.0;
  int iter = 0, lin_total = 0;
  while (iter < B.newton.max_its) {
    for (int f : B.fields) distribute(P.fields[f].cons, P.fields[f].cur.data());
    block_op(P, B, 0, nullptr, R.data());
    l2 = std::sqrt(dotp(R, R));
    if (!(l2 > tol)) break;
    if (B.lin.precond == 1) {  // fine-level diagonal of the current Jacobian
      OLevel& Lf = B.levels.back();
      compute_inv_diag(P, B, Lf.inv_diag);
      Lf.eig_done = false;
      estimate_eig(Lf, B);
    }
    bool lconv = false;
    double lres = 0.0;
    lin_total += block_krylov(P, B, R, B.newton_update, lin_tol, &lconv, &lres);
    for (int i = 0; i < nbf; ++i) {
      Field& F = P.fields[B.fields[i]];
      for (size_t j = 0; j < off[i + 1] - off[i]; ++j) F.cur[j] += B.newton.step * B.newton_update[off[i] + j];
    }
    ++iter;
  }
  B.last_newton_its = iter;
  B.last_newton_lin_its = lin_total;
  B.last_newton_res = l2 / norm;
  return iter >= B.newton.max_its ? 4 : 0;
}

Problem* make_problem(int dim, int degree, const int* subdiv, const double* lower, const double* size, int refine,
                      const int* periodic) {
  auto* P = new Problem();
  Mesh& m = P->m;
  m.dim = dim; m.k = degree; m.n = degree + 1;
  m.nloc = 1; for (int d = 0; d < dim; ++d) m.nloc *= m.n;
  int sd[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) { sd[d] = subdiv[d]; m.lo[d] = lower[d]; m.len[d] = size[d]; m.periodic[d] = periodic[d]; }
  for (int d = 0; d < 3; ++d) P->subdiv[d] = sd[d];
  P->refine = refine;
  build_cells(m, sd, refine);
  for (int d = 0; d < 3; ++d) {
    m.h[d] = d < dim ? m.len[d] / m.nc[d] : 1.0;
    m.nnode[d] = d < dim ? m.k * m.nc[d] + 1 : 1;
  }
  m.gl = make_gl(m.n);
  distribute_dofs(m, 0);
  distribute_dofs(m, 1);
  compute_invm(*P);
  return P;
}

// state vectors and constraints of every field; the number of old ages a field keeps is
// the oldest age any block depends on
void finalize_fields(Problem& P) {
  for (size_t f = 0; f < P.fields.size(); ++f) {
    Field& F = P.fields[f];
    const long nd = P.m.dh[F.rank].ndofs;
    int n_old = 0;
    for (auto& B : P.blocks)
      for (int a = AGE_OLD1; a <= AGE_OLD4; ++a)
        if (B.dep_rhs[f][a] || B.dep_lhs[f][a]) n_old = std::max(n_old, a);
    F.n_old = n_old;
    F.cur.assign(nd, 0.0);
    for (int a = 0; a < 4; ++a) F.old[a].assign(a < n_old ? nd : 0, 0.0);
    make_field_constraints(P, (int)f);
  }
}

// ---------------------------------------------------------------------------------------
// Adaptive meshes: RefinementManager (src/core/refinement_manager.cc:42-439) with deal.II's
// refinement smoothing, hanging-node constraints and SolutionTransfer, restated by brute
// force for small meshes (every geometric query scans all cells).
//
//  * A cell is (level l, integer coordinates i at level l); with M the maximum refinement
//    level it spans [i k, (i+1) k] 2^(M-l) in node units. Degrees 1 and 2: their Gauss-Lobatto
//    points (0, 1 / 0, 1/2, 1) nest under bisection, so node positions are the integers
//    (i k + a) 2^(M-l). Periodic positions wrap modulo the extent: a periodic image is the
//    same DoF as its master (the state deal.II's periodicity constraints distribute).
//  * Active cells are kept in tree order: coarse cells lexicographically (x fastest), the
//    children of a refined cell depth-first in lexicographic child order. DoFs are numbered
//    by first touch over that order, cell nodes lexicographically; vector fields are
//    component-major.
//  * A DoF is hanging when an active cell contains it without having it as a node; its line
//    is that cell's interpolant, weights prod_d L_a(xi_d), closed over chains
//    (DoFTools::make_hanging_node_constraints + AffineConstraints::close,
//    constraint_manager.cc:288-294). Dirichlet lines are added afterwards for boundary DoFs
//    that are not already constrained.
//  * The lumped mass condenses hanging nodes (hanging rows get invM = 0): the reference's
//    generic constraints hold periodicity only (constraint_manager.cc:156-170), but deal.II's
//    MatrixFree resolves hanging nodes from the mesh itself, so integrate_scatter in
//    InvMManager::compute_local_scalar (invm_manager.h:173-190) condenses them.
//  * Marking (refinement_manager.cc:161-363): a cell is flagged for refinement when any
//    criterion holds at any of its quadrature points (value in the open range; gradient
//    magnitude above the bound; vector fields by their l2 norms, the gradient of a vector
//    field compared with the value range as the reference does), below max refinement;
//    otherwise it is flagged for coarsening above min refinement.
//  * Smoothing, iterated to a fixed point (each rule only moves flags towards refinement,
//    so the result does not depend on the visiting order): coarsening only of complete
//    families of active, coarsening-flagged siblings; 2:1 balance between every two cells
//    that touch (share at least a vertex) after the change; an unrefined cell whose face
//    neighbours are mostly refined (finer, or flagged for refinement) is refined
//    (smoothing_on_refinement = limit_level_difference_at_vertices +
//    eliminate_unrefined_islands, triangulation_manager.cc:32-38).
//  * Transfer (group_solution_handler.cc:248-288): a node that existed before keeps its old
//    value; a new node takes the interpolant of the first old cell (in old order) that
//    contains it; then the new constraints are distributed on every age.
// ---------------------------------------------------------------------------------------
enum { REFINE_VALUE = 1, REFINE_GRADIENT = 2 };

static double lagrange_exact(int k, int a, double xi) {
  static const double q1[2] = {0.0, 1.0};
  static const double q2[3] = {0.0, 0.5, 1.0};
  const double* x = k == 1 ? q1 : q2;
  double v = 1.0;
  for (int b = 0; b <= k; ++b)
    if (b != a) v *= (xi - x[b]) / (x[a] - x[b]);
  return v;
}

static long span_w(const Mesh& m, long c) { return (long)m.k << (m.maxlev - m.lev[c]); }
static long span_lo(const Mesh& m, long c, int d) { return ((long)m.cells[c][d] * m.k) << (m.maxlev - m.lev[c]); }

static std::array<long, 3> node_position(const Mesh& m, long c, int l) {
  const int n = m.n;
  const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
  std::array<long, 3> P{0, 0, 0};
  for (int d = 0; d < m.dim; ++d) {
    long p = ((long)m.cells[c][d] * m.k + idx[d]) << (m.maxlev - m.lev[c]);
    if (m.periodic[d] && p == m.E[d]) p = 0;
    P[d] = p;
  }
  return P;
}

// offsets of position P inside the closure of cell c (periodic images unwrapped)
static bool local_offset(const Mesh& m, long c, const std::array<long, 3>& P, long* off) {
  const long w = span_w(m, c);
  for (int d = 0; d < m.dim; ++d) {
    const long lo = span_lo(m, c, d);
    long x = P[d];
    if (m.periodic[d] && x == 0 && lo + w == m.E[d]) x = m.E[d];
    if (x < lo || x > lo + w) return false;
    off[d] = x - lo;
  }
  return true;
}

static void adaptive_dofs(Mesh& m) {
  const int dim = m.dim, nloc = m.nloc;
  std::map<std::array<long, 3>, long> id;
  m.pos.clear();
  std::vector<long> cd((size_t)m.ncells * nloc);
  for (long c = 0; c < m.ncells; ++c)
    for (int l = 0; l < nloc; ++l) {
      const auto P = node_position(m, c, l);
      auto it = id.find(P);
      if (it == id.end()) {
        it = id.emplace(P, (long)m.pos.size()).first;
        m.pos.push_back(P);
      }
      cd[(size_t)c * nloc + l] = it->second;
    }
  const long N = (long)m.pos.size();
  for (int which = 0; which < 2; ++which) {
    DofHandler& d = m.dh[which];
    d.ncomp = which == 0 ? 1 : dim;
    d.ndofs = N * d.ncomp;
    d.cell_dofs.assign((size_t)m.ncells * d.ncomp * nloc, 0);
    d.lattice.assign(d.ndofs, {0, 0, 0, 0});
    for (long c = 0; c < m.ncells; ++c)
      for (int comp = 0; comp < d.ncomp; ++comp)
        for (int l = 0; l < nloc; ++l) d.cell_dofs[((size_t)c * d.ncomp + comp) * nloc + l] = comp * N + cd[(size_t)c * nloc + l];
    for (int comp = 0; comp < d.ncomp; ++comp)
      for (long i = 0; i < N; ++i)
        d.lattice[comp * N + i] = {(int)m.pos[i][0], (int)m.pos[i][1], (int)m.pos[i][2], comp};
  }
}

// hanging-node lines of the scalar DoFs, closed, entries in ascending master order
static void hanging_lines(Problem& P) {
  const Mesh& m = P.m;
  const long N = (long)m.pos.size();
  const int n = m.n, nloc = m.nloc;
  Constraints& H = P.hanging;
  H.reinit(N);
  for (long p = 0; p < N; ++p) {
    for (long c = 0; c < m.ncells; ++c) {
      long off[3] = {0, 0, 0};
      if (!local_offset(m, c, m.pos[p], off)) continue;
      const long step = 1L << (m.maxlev - m.lev[c]);
      bool node = true;
      for (int d = 0; d < m.dim; ++d) node &= (off[d] % step) == 0;
      if (node) continue;
      const double w = (double)span_w(m, c);
      H.add_line(p);
      for (int l = 0; l < nloc; ++l) {
        const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
        double wl = 1.0;
        for (int d = 0; d < m.dim; ++d) wl *= lagrange_exact(m.k, idx[d], off[d] / w);
        if (wl != 0.0) H.entries[p].push_back({m.dh[0].cell_dofs[(size_t)c * nloc + l], wl});
      }
      break;
    }
  }
  H.close();
  for (auto& e : H.entries) std::sort(e.begin(), e.end());
}

static bool on_boundary_pos(const Mesh& m, const std::array<long, 3>& P, int bid) {
  const int d = bid / 2;
  if (d >= m.dim || m.periodic[d]) return false;
  return (bid % 2 == 0) ? P[d] == 0 : P[d] == m.E[d];
}

static void make_field_constraints_adaptive(Problem& P, int f) {
  Field& F = P.fields[f];
  const Mesh& m = P.m;
  const DofHandler& d = m.dh[F.rank];
  const long N = (long)m.pos.size();
  F.cons.reinit(d.ndofs);
  for (int comp = 0; comp < d.ncomp; ++comp)
    for (long p = 0; p < N; ++p) {
      if (!P.hanging.is_constrained(p)) continue;
      const long i = comp * N + p;
      F.cons.add_line(i);
      for (auto& e : P.hanging.entries[p]) F.cons.entries[i].push_back({comp * N + e.first, e.second});
    }
  for (int comp = 0; comp < d.ncomp; ++comp)
    for (int bid = 0; bid < 2 * m.dim; ++bid) {
      if (!F.dir_on[comp][bid]) continue;
      for (long p = 0; p < N; ++p) {
        const long i = comp * N + p;
        if (!on_boundary_pos(m, m.pos[p], bid) || F.cons.is_constrained(i)) continue;
        F.cons.add_line(i);
        F.cons.inhom[i] = F.dir_val[comp][bid];
      }
    }
  F.cons.close();
}

// per-cell flags from the refinement criteria: 1 refine, -1 coarsen, 0 keep
static std::vector<int> mark_cells(Problem& P) {
  const Mesh& m = P.m;
  const int dim = m.dim, n = m.n, nloc = m.nloc;
  std::vector<int> flag(m.ncells, 0);
  std::vector<double> u((size_t)3 * nloc);
  for (long c = 0; c < m.ncells; ++c) {
    double hc[3];
    cell_h(m, c, hc);
    bool refine = false;
    for (const auto& K : P.criteria) {
      const Field& F = P.fields[K.field];
      const int ncomp = F.rank == 0 ? 1 : dim;
      const DofHandler& dh = m.dh[F.rank];
      for (int comp = 0; comp < ncomp; ++comp)
        for (int l = 0; l < nloc; ++l) u[comp * nloc + l] = F.cur[dh.cell_dofs[((size_t)c * ncomp + comp) * nloc + l]];
      for (int l = 0; l < nloc && !refine; ++l) {
        if (K.flags & REFINE_VALUE) {
          double v;
          if (ncomp == 1) v = u[l];
          else {
            double s2 = 0.0;
            for (int comp = 0; comp < ncomp; ++comp) s2 += u[comp * nloc + l] * u[comp * nloc + l];
            v = std::sqrt(s2);
          }
          if (v > K.vlo && v < K.vhi) refine = true;
        }
        if (!refine && (K.flags & REFINE_GRADIENT)) {
          const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
          const int stride[3] = {1, n, n * n};
          double mag2 = 0.0;
          for (int comp = 0; comp < ncomp; ++comp) {
            double g2 = 0.0;
            for (int d = 0; d < dim; ++d) {
              const int base = l - idx[d] * stride[d];
              double acc = 0.0;
              for (int j = 0; j < n; ++j) acc += m.gl.D[idx[d]][j] * u[comp * nloc + base + j * stride[d]];
              const double g = acc / hc[d];
              g2 += g * g;
            }
            if (ncomp == 1) mag2 = g2;
            else {
              const double gm = std::sqrt(g2);
              mag2 += gm * gm;
            }
          }
          const double mag = std::sqrt(mag2);
          if (ncomp == 1 ? mag > K.glo : (mag > K.vlo && mag < K.vhi)) refine = true;
        }
      }
      if (refine) break;
    }
    if (refine) flag[c] = m.lev[c] < P.max_level ? 1 : 0;
    else flag[c] = m.lev[c] > P.min_level ? -1 : 0;
  }
  return flag;
}

static bool overlap(long a0, long a1, long b0, long b1) { return a0 <= b1 && b0 <= a1; }
static bool open_overlap(long a0, long a1, long b0, long b1) { return a0 < b1 && b0 < a1; }

// closures of cells a and b intersect (periodic directions wrap)
static bool cells_touch(const Mesh& m, long a, long b) {
  const long wa = span_w(m, a), wb = span_w(m, b);
  for (int d = 0; d < m.dim; ++d) {
    const long a0 = span_lo(m, a, d), b0 = span_lo(m, b, d);
    bool hit = overlap(a0, a0 + wa, b0, b0 + wb);
    if (!hit && m.periodic[d])
      hit = overlap(a0, a0 + wa, b0 + m.E[d], b0 + wb + m.E[d]) || overlap(a0, a0 + wa, b0 - m.E[d], b0 + wb - m.E[d]);
    if (!hit) return false;
  }
  return true;
}

// b lies across face (dir, side) of a: touches that face and overlaps it with positive measure
static bool across_face(const Mesh& m, long a, long b, int dir, int side) {
  const long wa = span_w(m, a), wb = span_w(m, b);
  for (int d = 0; d < m.dim; ++d) {
    const long a0 = span_lo(m, a, d), b0 = span_lo(m, b, d);
    bool ok = false;
    for (int sh = -1; sh <= 1 && !ok; ++sh) {
      if (sh != 0 && !m.periodic[d]) continue;
      const long s0 = b0 + sh * m.E[d];
      if (d == dir) ok = side ? s0 == a0 + wa : s0 + wb == a0;
      else ok = open_overlap(a0, a0 + wa, s0, s0 + wb);
    }
    if (!ok) return false;
  }
  return true;
}

typedef std::array<int, 4> CellKey;  // level, i, j, k

static CellKey parent_key(const Mesh& m, long c) {
  return {m.lev[c] - 1, m.cells[c][0] >> 1, m.cells[c][1] >> 1, m.cells[c][2] >> 1};
}

// refinement smoothing of the flags to a fixed point
static void smooth_flags(Problem& P, std::vector<int>& flag) {
  const Mesh& m = P.m;
  const long nc = m.ncells;
  const int nchild = 1 << m.dim;
  for (;;) {
    bool changed = false;
    std::map<CellKey, int> fam;
    for (long c = 0; c < nc; ++c)
      if (flag[c] == -1) fam[parent_key(m, c)]++;
    for (long c = 0; c < nc; ++c)
      if (flag[c] == -1 && fam[parent_key(m, c)] != nchild) { flag[c] = 0; changed = true; }
    for (long a = 0; a < nc; ++a) {
      const int ta = m.lev[a] + (flag[a] == 1) - (flag[a] == -1);
      for (long b = 0; b < nc; ++b) {
        if (a == b) continue;
        const int tb = m.lev[b] + (flag[b] == 1) - (flag[b] == -1);
        if (ta <= tb + 1 || !cells_touch(m, a, b)) continue;
        const int nf = flag[b] == -1 ? 0 : 1;
        if (nf != flag[b]) {
          flag[b] = nf;
          changed = true;
        }
      }
    }
    for (long a = 0; a < nc; ++a) {
      if (flag[a] == 1) continue;
      int refined = 0, unrefined = 0;
      for (int dir = 0; dir < m.dim; ++dir)
        for (int side = 0; side < 2; ++side) {
          bool any = false, fine = false;
          for (long b = 0; b < nc; ++b) {
            if (b == a || !across_face(m, a, b, dir, side)) continue;
            any = true;
            if (m.lev[b] > m.lev[a] || (m.lev[b] == m.lev[a] && flag[b] == 1)) fine = true;
          }
          if (!any) continue;  // domain boundary
          if (fine) ++refined;
          else ++unrefined;
        }
      if (refined > unrefined && m.lev[a] < P.max_level) {
        flag[a] = 1;
        changed = true;
      }
    }
    if (!changed) break;
  }
}

static void tree_order(const Mesh& m, const std::map<CellKey, CellKey>& act, int l, int i, int j, int k,
                       std::vector<CellKey>& out) {
  auto it = act.find(CellKey{l, i, j, k});
  if (it != act.end()) {
    out.push_back(it->second);
    return;
  }
  if (l >= m.maxlev) return;
  for (int ch = 0; ch < (1 << m.dim); ++ch)
    tree_order(m, act, l + 1, 2 * i + (ch & 1), 2 * j + ((ch >> 1) & 1), m.dim == 3 ? 2 * k + ((ch >> 2) & 1) : 0, out);
}

static void set_cells(Mesh& m, const std::vector<CellKey>& cells) {
  std::map<CellKey, CellKey> act;
  for (auto& c : cells) act[c] = c;
  std::vector<CellKey> ordered;
  for (int k = 0; k < (m.dim == 3 ? m.sub[2] : 1); ++k)
    for (int j = 0; j < m.sub[1]; ++j)
      for (int i = 0; i < m.sub[0]; ++i) tree_order(m, act, 0, i, j, k, ordered);
  m.ncells = (long)ordered.size();
  m.cells.resize(m.ncells);
  m.lev.resize(m.ncells);
  for (long c = 0; c < m.ncells; ++c) {
    m.lev[c] = ordered[c][0];
    m.cells[c] = {ordered[c][1], ordered[c][2], ordered[c][3]};
  }
}

static void rebuild_mesh(Problem& P) {
  adaptive_dofs(P.m);
  hanging_lines(P);
  compute_invm(P);
  for (size_t f = 0; f < P.fields.size(); ++f) make_field_constraints(P, (int)f);
}

// one remesh pass (RefinementManager::do_adaptive_refinement): mark, smooth, refine/coarsen,
// renumber, transfer every stored age, distribute the new constraints
static void remesh_with_flags(Problem& P, std::vector<int> flag);

static void remesh(Problem& P) { remesh_with_flags(P, mark_cells(P)); }

// the pass from given marks (1 refine, -1 coarsen, 0 keep) on: smoothing, refine/coarsen,
// renumbering, transfer
static void remesh_with_flags(Problem& P, std::vector<int> flag) {
  Mesh& m = P.m;
  smooth_flags(P, flag);
  std::vector<CellKey> nxt;
  std::map<CellKey, int> parents_done;
  for (long c = 0; c < m.ncells; ++c) {
    const int l = m.lev[c];
    const auto& x = m.cells[c];
    if (flag[c] == 1) {
      for (int ch = 0; ch < (1 << m.dim); ++ch)
        nxt.push_back({l + 1, 2 * x[0] + (ch & 1), 2 * x[1] + ((ch >> 1) & 1), m.dim == 3 ? 2 * x[2] + ((ch >> 2) & 1) : 0});
    } else if (flag[c] == -1) {
      if (parents_done[parent_key(m, c)]++ == 0) nxt.push_back({l - 1, x[0] >> 1, x[1] >> 1, x[2] >> 1});
    } else {
      nxt.push_back({l, x[0], x[1], x[2]});
    }
  }
  const Mesh old = m;
  set_cells(m, nxt);
  rebuild_mesh(P);
  // transfer plan per new scalar DoF: (old dof, weight) entries
  std::map<std::array<long, 3>, long> oldpos;
  for (long i = 0; i < (long)old.pos.size(); ++i) oldpos[old.pos[i]] = i;
  const long N = (long)m.pos.size(), No = (long)old.pos.size();
  const int n = m.n, nloc = m.nloc;
  std::vector<std::vector<std::pair<long, double>>> plan(N);
  for (long p = 0; p < N; ++p) {
    auto it = oldpos.find(m.pos[p]);
    if (it != oldpos.end()) {
      plan[p].push_back({it->second, 1.0});
      continue;
    }
    for (long c = 0; c < old.ncells; ++c) {
      long off[3] = {0, 0, 0};
      if (!local_offset(old, c, m.pos[p], off)) continue;
      const double w = (double)span_w(old, c);
      for (int l = 0; l < nloc; ++l) {
        const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
        double wl = 1.0;
        for (int d = 0; d < m.dim; ++d) wl *= lagrange_exact(m.k, idx[d], off[d] / w);
        if (wl != 0.0) plan[p].push_back({old.dh[0].cell_dofs[(size_t)c * nloc + l], wl});
      }
      break;
    }
  }
  for (auto& F : P.fields) {
    const int ncomp = F.rank == 0 ? 1 : m.dim;
    auto move = [&](std::vector<double>& v) {
      if (v.empty()) return;
      std::vector<double> nv((size_t)ncomp * N, 0.0);
      for (int comp = 0; comp < ncomp; ++comp)
        for (long p = 0; p < N; ++p) {
          double s = 0.0;
          for (auto& e : plan[p]) s += e.second * v[comp * No + e.first];
          nv[comp * N + p] = s;
        }
      distribute(F.cons, nv.data());
      v.swap(nv);
    };
    move(F.cur);
    for (int a = 0; a < F.n_old; ++a) move(F.old[a]);
  }
  // linear and Newton solvers start over on the new mesh (warm starts from zero)
  for (auto& B : P.blocks) {
    for (auto& L : B.levels)
      if (L.owned) delete L.P;
    B.levels.clear();
    B.lin_init = false;
    B.x_hom.clear();
    B.newton_update.clear();
  }
}

static int enable_adaptivity(Problem& P, int min_level, int max_level, int period) {
  Mesh& m = P.m;
  if (m.dim < 2 || m.k > 2 || min_level < 0 || max_level < P.refine || min_level > P.refine || max_level > 18)
    return -1;
  for (int d = 0; d < m.dim; ++d)
    if (m.periodic[d] && ((long)P.subdiv[d] << min_level) < 2) return -1;
  m.adaptive = true;
  m.maxlev = max_level;
  for (int d = 0; d < 3; ++d) {
    m.sub[d] = P.subdiv[d];
    m.E[d] = d < m.dim ? ((long)m.sub[d] * m.k) << max_level : 1;
  }
  m.lev.assign(m.ncells, P.refine);
  std::vector<CellKey> cells;
  for (long c = 0; c < m.ncells; ++c) cells.push_back({P.refine, m.cells[c][0], m.cells[c][1], m.cells[c][2]});
  set_cells(m, cells);
  P.min_level = min_level;
  P.max_level = max_level;
  P.period = period;
  rebuild_mesh(P);
  return 0;
}

// the refinement step of Problem::solve_increment (problem.cc:488-499): at increment 0 up to
// max - min passes, stopping when the DoF count no longer changes; later every `period`
// increments one pass
static void remesh_if_due(Problem& P) {
  if (!P.m.adaptive) return;
  if (P.increment == 0) {
    for (int r = 0; r < P.max_level - P.min_level; ++r) {
      const size_t n0 = P.m.pos.size();
      remesh(P);
      if (P.m.pos.size() == n0) break;
    }
  } else if (P.period > 0 && P.increment % (unsigned)P.period == 0) {
    remesh(P);
  }
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------------------
extern "C" {

void* orc_create(int dim, int degree, const int* subdiv, const double* lower, const double* size,
                 int refine, const int* periodic) {
  if (dim < 1 || dim > 3 || degree < 1 || degree > 6) return nullptr;
  return make_problem(dim, degree, subdiv, lower, size, refine, periodic);
}

void orc_destroy(void* h) { delete (Problem*)h; }

void orc_set_threads(void* h, int n) { ((Problem*)h)->nthreads = n; }

long orc_n_dofs(void* h, int rank) { return ((Problem*)h)->m.dh[rank].ndofs; }
long orc_n_cells(void* h) { return ((Problem*)h)->m.ncells; }

void orc_gl(int n, double* x, double* w, double* D) {
  GL g = make_gl(n);
  for (int i = 0; i < n; ++i) { x[i] = g.x[i]; w[i] = g.w[i]; for (int j = 0; j < n; ++j) D[i * n + j] = g.D[i][j]; }
}

void orc_lattice(void* h, int rank, int* out) {
  auto& d = ((Problem*)h)->m.dh[rank];
  for (long i = 0; i < d.ndofs; ++i) for (int k = 0; k < 4; ++k) out[i * 4 + k] = d.lattice[i][k];
}

void orc_cell_dofs(void* h, int rank, long* out) {
  auto& d = ((Problem*)h)->m.dh[rank];
  std::memcpy(out, d.cell_dofs.data(), d.cell_dofs.size() * sizeof(long));
}

void orc_cell_coords(void* h, int* out) {
  auto& m = ((Problem*)h)->m;
  for (long c = 0; c < m.ncells; ++c) for (int k = 0; k < 3; ++k) out[c * 3 + k] = m.cells[c][k];
}

void orc_invm(void* h, int rank, double* out) {
  auto* P = (Problem*)h;
  std::memcpy(out, P->invm[rank].data(), P->invm[rank].size() * sizeof(double));
}

int orc_add_field(void* h, int rank) {
  auto* P = (Problem*)h;
  Field F; F.rank = rank;
  P->fields.push_back(F);
  return (int)P->fields.size() - 1;
}

void orc_set_dirichlet(void* h, int field, int comp, int boundary_id, double value) {
  auto* P = (Problem*)h;
  P->fields[field].dir_on[comp][boundary_id] = 1;
  P->fields[field].dir_val[comp][boundary_id] = value;
}

// deps: nfields * 6 flags (ages: current, old1..old4, src) for rhs then lhs
int orc_add_block(void* h, int id, int solve_type, int timing, const int* fields, int nf,
                  const int* dep_rhs, const int* dep_lhs) {
  auto* P = (Problem*)h;
  Block B; B.id = id; B.solve_type = solve_type; B.timing = timing;
  for (int i = 0; i < nf; ++i) B.fields.push_back(fields[i]);
  const int NF = (int)P->fields.size();
  B.dep_rhs.assign(NF, {}); B.dep_lhs.assign(NF, {});
  for (int f = 0; f < NF; ++f)
    for (int a = 0; a < NAGE; ++a) {
      B.dep_rhs[f][a] = dep_rhs ? dep_rhs[f * NAGE + a] : 0;
      B.dep_lhs[f][a] = dep_lhs ? dep_lhs[f * NAGE + a] : 0;
    }
  P->blocks.push_back(B);
  return (int)P->blocks.size() - 1;
}

int orc_finalize(void* h, int model, const double* params, int nparams, double dt) {
  auto* P = (Problem*)h;
  P->model = model;
  P->params.assign(params, params + nparams);
  P->dt = dt;
  if (!callback_for(model)) return -1;
  finalize_fields(*P);
  return 0;
}

// constraint export: kind (0 free, 1 constrained), master (first entry or -1), inhomogeneity
void orc_constraints(void* h, int field, int* kind, long* master, double* inhom) {
  auto* P = (Problem*)h;
  auto& C = P->fields[field].cons;
  for (size_t i = 0; i < C.constrained.size(); ++i) {
    kind[i] = C.constrained[i];
    master[i] = (C.constrained[i] && !C.entries[i].empty()) ? C.entries[i][0].first : -1;
    inhom[i] = C.inhom[i];
  }
}

int orc_set_vector(void* h, int field, int age, const double* v) {
  auto* P = (Problem*)h;
  Field& F = P->fields[field];
  std::vector<double>& dst = age == 0 ? F.cur : F.old[age - 1];
  if (dst.empty()) return -1;
  std::memcpy(dst.data(), v, dst.size() * sizeof(double));
  return 0;
}

int orc_get_vector(void* h, int field, int age, double* v) {
  auto* P = (Problem*)h;
  Field& F = P->fields[field];
  std::vector<double>& src = age == 0 ? F.cur : F.old[age - 1];
  if (src.empty()) return -1;
  std::memcpy(v, src.data(), src.size() * sizeof(double));
  return 0;
}

void orc_set_time(void* h, unsigned increment, double time) {
  auto* P = (Problem*)h;
  P->increment = increment; P->time = time;
}

// One explicit solve of block index b (ExplicitSolver::solve_impl)
int orc_explicit_block(void* h, int b) {
  auto* P = (Problem*)h;
  explicit_solve(*P, P->blocks[b]);
  return 0;
}

// The Problem::solve increment loop (explicit blocks only); output_every > 0 makes
// PostProcess blocks run on increments that are multiples of it.
// Block b's part of the current increment (Problem::solve_increment, problem.cc:416-557).
int orc_increment_block(void* h, int b, int is_output) {
  auto* P = (Problem*)h;
  Block& B = P->blocks[b];
  // PostProcess only on output increments; NucleationRate on output and nucleation-attempt
  // increments (problem.cc:436-443)
  if (B.timing == ORC_TIMING_POSTPROCESS && !is_output) return 0;
  if (B.timing == ORC_TIMING_NUCLEATION_RATE && !is_output && P->increment % P->nucleation_period != 0) return 0;
  if (P->increment == 0 && B.timing == ORC_TIMING_PRIMARY) {
    // initial condition already uploaded into `cur`; like
    // SolverBase::set_initial_condition (solver_base.h:178-229) no constraints are
    // distributed on it at increment 0
  } else {
    if (B.solve_type == 2) linear_solve(*P, B);
    else if (B.solve_type == 3) {
      const int rc = newton_solve(*P, B);
      if (rc != 0 && rc != 4) return rc;  // non-convergence is a warning in the reference
    } else explicit_solve(*P, B);
  }
  if (P->increment == 0) {
    for (int f : B.fields) {
      Field& F = P->fields[f];
      for (int a = 0; a < F.n_old; ++a) F.old[a] = F.cur;
    }
  }
  return 0;
}

int orc_set_nucleation_period(void* h, unsigned period) {
  if (period < 1) return -1;
  static_cast<Problem*>(h)->nucleation_period = period;
  return 0;
}

// End of an increment: NaN check, rotation by swap (group_solution_handler.cc:369-403), time.
int orc_end_increment(void* h) {
  auto* P = (Problem*)h;
  for (auto& F : P->fields)
    if (!std::isfinite(F.cur.empty() ? 0.0 : F.cur[0])) return ORC_ERR_NAN;
  for (auto& F : P->fields)
    for (int age = F.n_old - 1; age >= 0; --age) {
      if (age > 0) F.old[age].swap(F.old[age - 1]);
      else F.old[0].swap(F.cur);
    }
  P->increment++;
  P->time += P->dt;
  return 0;
}

// The Problem::solve increment loop; output_every > 0 makes PostProcess blocks run on
// increments that are multiples of it.
int orc_run(void* h, unsigned n_increments, int output_every) {
  auto* P = (Problem*)h;
  while (P->increment <= n_increments) {
    const int is_output = output_every > 0 && (P->increment % (unsigned)output_every) == 0;
    for (size_t b = 0; b < P->blocks.size(); ++b) {
      const int rc = orc_increment_block(h, (int)b, is_output);
      if (rc) return rc;
    }
    remesh_if_due(*P);
    const int rc = orc_end_increment(h);
    if (rc) return rc;
  }
  return 0;
}

// ---- adaptive meshes -------------------------------------------------------------------
// Mesh adaptivity (SpatialDiscretization::has_adaptivity): call after the fields are added
// and before orc_finalize. criteria: n entries of (field, flags 1 value | 2 gradient, value
// lower, value upper, gradient lower). The mesh starts uniform at the global refinement.
int orc_set_adaptivity(void* h, int min_level, int max_level, int period, int n, const int* fields,
                       const int* flags, const double* vlo, const double* vhi, const double* glo) {
  auto* P = (Problem*)h;
  P->criteria.clear();
  for (int i = 0; i < n; ++i) P->criteria.push_back({fields[i], flags[i], vlo[i], vhi[i], glo[i]});
  return enable_adaptivity(*P, min_level, max_level, period);
}

// one remesh pass (mark, smooth, refine/coarsen, transfer)
int orc_adapt(void* h) {
  auto* P = (Problem*)h;
  if (!P->m.adaptive) return -1;
  remesh(*P);
  return 0;
}

// one remesh pass from given per-cell marks (tree order; 1 refine, -1 coarsen, 0 keep) in
// place of the refinement criteria
int orc_adapt_with_flags(void* h, const int* flags) {
  auto* P = (Problem*)h;
  if (!P->m.adaptive) return -1;
  remesh_with_flags(*P, std::vector<int>(flags, flags + P->m.ncells));
  return 0;
}

// the refinement step of the current increment, as orc_run does it after the blocks
int orc_remesh_if_due(void* h) {
  remesh_if_due(*(Problem*)h);
  return 0;
}

long orc_n_nodes(void* h) {
  auto* P = (Problem*)h;
  return P->m.adaptive ? (long)P->m.pos.size() : P->m.dh[0].ndofs;
}

// active cells in tree order: level, i, j, k per cell
void orc_cells(void* h, int* out) {
  auto& m = ((Problem*)h)->m;
  for (long c = 0; c < m.ncells; ++c) {
    out[c * 4] = m.adaptive ? m.lev[c] : ((Problem*)h)->refine;
    for (int d = 0; d < 3; ++d) out[c * 4 + 1 + d] = m.cells[c][d];
  }
}

// coordinates of the scalar DoFs of an adaptive mesh: lower + size * (position / extent)
void orc_node_points(void* h, double* out) {
  auto& m = ((Problem*)h)->m;
  for (size_t i = 0; i < m.pos.size(); ++i)
    for (int d = 0; d < 3; ++d) out[i * 3 + d] = d < m.dim ? m.lo[d] + m.len[d] * ((double)m.pos[i][d] / (double)m.E[d]) : 0.0;
}

// closed hanging-node lines of the scalar DoFs: per DoF the entry count (0 when free), then
// the entries (master, weight) in ascending master order. Returns the total entry count;
// call with null outputs to size them.
long orc_hanging(void* h, int* count, long* master, double* weight) {
  auto& H = ((Problem*)h)->hanging;
  long t = 0;
  for (size_t i = 0; i < H.constrained.size(); ++i) {
    const long c = H.constrained[i] ? (long)H.entries[i].size() : 0;
    if (count) count[i] = (int)c;
    if (H.constrained[i])
      for (auto& e : H.entries[i]) {
        if (master) master[t] = e.first;
        if (weight) weight[t] = e.second;
        ++t;
      }
  }
  return t;
}

// Operator apply of block b: which = 0 rhs (plain read), 1 lhs (src read with constraints).
// src/dst are per block-field vectors concatenated in block field order. scale: 0 none,
// 1 invM, 2 invM^1/2.
int orc_apply(void* h, int b, int which, const double* src, double* dst, int scale) {
  auto* P = (Problem*)h;
  Block& B = P->blocks[b];
  std::vector<const double*> s;
  std::vector<double*> d;
  std::vector<const Constraints*> cons;
  size_t off = 0;
  for (int f : B.fields) {
    Field& F = P->fields[f];
    const size_t nd = F.cur.size();
    s.push_back(src ? src + off : nullptr);
    std::fill(dst + off, dst + off + nd, 0.0);
    d.push_back(dst + off);
    cons.push_back(&F.cons);
    off += nd;
  }
  cell_loop(*P, B, which == 1, s, d, cons, callback_for(P->model));
  off = 0;
  for (int f : B.fields) {
    Field& F = P->fields[f];
    const size_t nd = F.cur.size();
    if (scale == 1) for (size_t i = 0; i < nd; ++i) dst[off + i] *= P->invm[F.rank][i];
    if (scale == 2) for (size_t i = 0; i < nd; ++i) dst[off + i] *= P->invm_sqrt[F.rank][i];
    off += nd;
  }
  return 0;
}

// Linear solver parameters of block b: p = {tol_type, tol, max_its, precond, mg_depth,
// degree, smoothing range, eig_its}
int orc_set_linear_params(void* h, int b, const double* p) {
  auto* P = (Problem*)h;
  LinParams& L = P->blocks[b].lin;
  L.tol_type = (int)p[0]; L.tol = p[1]; L.max_its = (int)p[2]; L.precond = (int)p[3];
  L.mg_depth = (int)p[4]; L.degree = (int)p[5]; L.range = p[6]; L.eig_its = (int)p[7];
  return 0;
}

int orc_set_solver_type(void* h, int b, int solver) {
  ((Problem*)h)->blocks[b].lin.solver = solver;
  return 0;
}

int orc_set_newton_params(void* h, int b, int max_its, double tol, double step) {
  NewtonParams& N = ((Problem*)h)->blocks[b].newton;
  N.max_its = max_its;
  N.tol = tol;
  N.step = step;
  return 0;
}

// One Newton solve of block b; its = Newton iterations, lin_its = total Krylov iterations,
// res = final residual norm / normalization
int orc_newton_solve(void* h, int b, int* its, int* lin_its, double* res) {
  auto* P = (Problem*)h;
  Block& B = P->blocks[b];
  const int rc = newton_solve(*P, B);
  if (its) *its = B.last_newton_its;
  if (lin_its) *lin_its = B.last_newton_lin_its;
  if (res) *res = B.last_newton_res;
  return rc;
}

int orc_linear_solve(void* h, int b, int* its, double* res) {
  auto* P = (Problem*)h;
  int rc = linear_solve(*P, P->blocks[b]);
  if (its) *its = P->blocks[b].last_its;
  if (res) *res = P->blocks[b].last_res;
  return rc;
}

// matrix diagonal of block b's LHS (scaled, zero entries one), deal.II order
void orc_diagonal(void* h, int b, double* out) {
  auto* P = (Problem*)h;
  std::vector<double> inv;
  compute_inv_diag(*P, P->blocks[b], inv);
  for (size_t i = 0; i < inv.size(); ++i) out[i] = 1.0 / inv[i];
}

}  // extern "C"
