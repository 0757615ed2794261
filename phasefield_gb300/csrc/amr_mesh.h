// Adaptive mesh of the engine (host side): a forest of quadtrees / octrees over the coarse
// subdivided rectangle, its DoF numbering, hanging-node constraints, refinement smoothing and
// the solution-transfer plan. Restates what PRISMS-PF's RefinementManager
// (src/core/refinement_manager.cc:42-439) asks of deal.II (p4est triangulation with
// smoothing_on_refinement, triangulation_manager.cc:32-38; DoFHandler::distribute_dofs;
// DoFTools::make_hanging_node_constraints, constraint_manager.cc:288-294; SolutionTransfer,
// group_solution_handler.cc:248-288) with hash lookups instead of cell scans:
//
//  * A cell is (level l, integer coordinates at level l); with M the maximum level it spans
//    [x k, (x+1) k] 2^(M-l) in node units. Degrees 1 and 2 only: their Gauss-Lobatto points
//    (0,1 and 0,1/2,1) nest under bisection, so node positions are exact integers and the
//    hanging-node weights are exact binary fractions.
//  * Active cells are kept in tree order (coarse cells lexicographic with x fastest, children
//    depth-first in lexicographic child order); DoFs are numbered by first touch over that
//    order with lexicographic cell nodes. Periodic positions wrap, so a periodic image is the
//    same DoF as its master.
//  * A DoF is hanging when an active cell contains it without having it as a node; it is
//    constrained to that cell's interpolant, closed over chains of hanging masters.
//  * Smoothing, iterated to a fixed point: coarsening only of complete families, 2:1 balance
//    between cells that share at least a vertex, refinement of unrefined islands (cells whose
//    face neighbours are mostly refined or flagged for refinement).
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace ppf {

struct AmrCell {
  int lev;
  int x[3];
};

// 64-bit key -> int table with open addressing (linear probing, power-of-two capacity at most
// half full); keys are cell and position keys, which never use the all-ones pattern.
class KeyTable {
 public:
  void reset(size_t expected);  // empties the table, sized for `expected` keys
  int find(uint64_t key) const;  // value or -1
  // the value stored for `key`, or `value` after inserting it (inserted tells which)
  int insert(uint64_t key, int value, bool& inserted);

 private:
  static constexpr uint64_t EMPTY = ~0ULL;
  void grow();
  std::vector<uint64_t> keys_;
  std::vector<int> vals_;
  uint64_t mask_ = 0;
  size_t count_ = 0;
};

struct AmrMesh {
  int dim = 2, k = 1, n = 2, nq = 4;
  int sub[3] = {1, 1, 1};
  int periodic[3] = {0, 0, 0};
  int maxlev = 0;
  long long E[3] = {1, 1, 1};                 // extent in node units at level maxlev
  std::vector<AmrCell> cells;                 // active cells in tree order
  KeyTable index;                             // cell key -> active cell index
  long long N = 0;                            // DoFs (nodes)
  std::vector<int> cell_dofs;                 // ncells * nq, lexicographic cell nodes
  std::vector<std::array<long long, 3>> pos;  // node position of every DoF
  KeyTable node_of;                           // position key -> DoF
  // closed hanging-node lines: row r constrains DoF h_dof[r] to
  // sum_{e in [h_ptr[r], h_ptr[r+1])} h_w[e] * u[h_idx[e]] (masters ascending, none hanging)
  std::vector<int> hang_row;                  // per DoF: its row or -1
  std::vector<int> h_dof, h_ptr, h_idx;
  std::vector<double> h_w;

  long long ncells() const { return (long long)cells.size(); }
  uint64_t cell_key(int lev, long long x, long long y, long long z) const;
  uint64_t pos_key(const std::array<long long, 3>& p) const;
  int find(int lev, long long x, long long y, long long z) const;  // active index or -1
};

// A uniform mesh at `level` (the global refinement); false with a message when the sizes do
// not fit the position encoding.
bool amr_init_uniform(AmrMesh& m, int dim, int degree, const int* subdivisions, const int* periodic, int level,
                      int max_level, std::string& err);

// DoF numbering, node positions and hanging-node lines of the current cells.
void amr_build(AmrMesh& m);

// Refinement smoothing of per-cell flags (1 refine, -1 coarsen, 0 keep) to a fixed point.
void amr_smooth(const AmrMesh& m, std::vector<signed char>& flags, int max_level);

// The cells after applying smoothed flags (the caller then calls amr_set_cells + amr_build).
std::vector<AmrCell> amr_refine(const AmrMesh& m, const std::vector<signed char>& flags);

// Replaces the cells of `m` (sorted into tree order) and rebuilds the index.
void amr_set_cells(AmrMesh& m, std::vector<AmrCell> cells);

// Transfer plan from `old` to `m`: new DoF p = sum_{e in [ptr[p], ptr[p+1])} w[e] old[idx[e]]
// (a node that existed keeps its value; a new node takes the interpolant of the first old
// cell containing it).
void amr_transfer_plan(const AmrMesh& old, const AmrMesh& m, std::vector<int>& ptr, std::vector<int>& idx,
                       std::vector<double>& w);

// Position of DoF p: lower + size * (position / extent).
void amr_point(const AmrMesh& m, const double* lower, const double* size, long long p, double* x);

}  // namespace ppf
