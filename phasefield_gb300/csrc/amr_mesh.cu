// Host-side adaptive mesh (forest of quadtrees / octrees): see amr_mesh.h.
#include "amr_mesh.h"

#include <algorithm>
#include <functional>
#include <unordered_set>

namespace ppf {

namespace {

constexpr int KEY_BITS = 19;  // cell coordinates per axis at any level: < 2^19
constexpr int POS_BITS = 21;  // node positions per axis: < 2^21

double lagrange_exact(int k, int a, double xi) {
  static const double q1[2] = {0.0, 1.0};
  static const double q2[3] = {0.0, 0.5, 1.0};
  const double* x = k == 1 ? q1 : q2;
  double v = 1.0;
  for (int b = 0; b <= k; ++b)
    if (b != a) v *= (xi - x[b]) / (x[a] - x[b]);
  return v;
}

long long cells_along(const AmrMesh& m, int d, int lev) { return (long long)m.sub[d] << lev; }

// wraps a coordinate at level lev along d; false when it leaves a non-periodic domain
bool wrap(const AmrMesh& m, int d, int lev, long long& x) {
  const long long n = cells_along(m, d, lev);
  if (x >= 0 && x < n) return true;
  if (!m.periodic[d]) return false;
  x = ((x % n) + n) % n;
  return true;
}

// offsets of position p inside the closure of a cell (periodic images unwrapped)
bool local_offset(const AmrMesh& m, int lev, const int* x, const std::array<long long, 3>& p, long long* off) {
  const long long w = (long long)m.k << (m.maxlev - lev);
  for (int d = 0; d < m.dim; ++d) {
    const long long lo = (long long)x[d] * w;
    long long q = p[d];
    if (m.periodic[d] && q == 0 && lo + w == m.E[d]) q = m.E[d];
    if (q < lo || q > lo + w) return false;
    off[d] = q - lo;
  }
  return true;
}

// active cells covering the region of level-`lev` cell y next to the asking cell: the region
// itself when active, else its active ancestor, else the active descendants on the side facing
// the asker (`dir` points from the region towards the asker)
void covering(const AmrMesh& m, int lev, long long y0, long long y1, long long y2, const int* dir,
              std::vector<int>& out) {
  const int i = m.find(lev, y0, y1, y2);
  if (i >= 0) {
    out.push_back(i);
    return;
  }
  for (int l = lev - 1; l >= 0; --l) {
    const int s = lev - l;
    const int a = m.find(l, y0 >> s, y1 >> s, y2 >> s);
    if (a >= 0) {
      out.push_back(a);
      return;
    }
  }
  if (lev >= m.maxlev) return;
  const long long y[3] = {y0, y1, y2};
  for (int ch = 0; ch < (1 << m.dim); ++ch) {
    long long c[3] = {0, 0, 0};
    bool ok = true;
    for (int d = 0; d < m.dim; ++d) {
      const int b = (ch >> d) & 1;
      if (dir[d] > 0 && b != 1) ok = false;  // the asker lies above the region: upper children
      if (dir[d] < 0 && b != 0) ok = false;  // below: lower children
      c[d] = 2 * y[d] + b;
    }
    if (ok) covering(m, lev + 1, c[0], c[1], c[2], dir, out);
  }
}

// active cells touching cell c (sharing at least a vertex); with face_axis >= 0 only the cells
// across face (face_axis, face_side)
void touching(const AmrMesh& m, int c, std::vector<int>& out, int face_axis = -1, int face_side = 0) {
  out.clear();
  const AmrCell& C = m.cells[c];
  const int nd = m.dim;
  int total = 1;
  for (int d = 0; d < nd; ++d) total *= 3;
  for (int t = 0; t < total; ++t) {
    int delta[3] = {0, 0, 0};
    int r = t;
    bool zero = true;
    for (int d = 0; d < nd; ++d) {
      delta[d] = r % 3 - 1;
      r /= 3;
      zero &= delta[d] == 0;
    }
    if (zero) continue;
    if (face_axis >= 0) {
      bool ok = true;
      for (int d = 0; d < nd; ++d) ok &= d == face_axis ? delta[d] == (face_side ? 1 : -1) : delta[d] == 0;
      if (!ok) continue;
    }
    long long y[3] = {0, 0, 0};
    bool inside = true;
    for (int d = 0; d < nd; ++d) {
      y[d] = (long long)C.x[d] + delta[d];
      inside &= wrap(m, d, C.lev, y[d]);
    }
    if (!inside) continue;
    const int back[3] = {-delta[0], -delta[1], -delta[2]};
    covering(m, C.lev, y[0], y[1], y[2], back, out);
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  out.erase(std::remove(out.begin(), out.end(), c), out.end());
}

uint64_t path_key(const AmrMesh& m, const AmrCell& c) {
  uint64_t key = 0;
  for (int t = 1; t <= m.maxlev; ++t) {
    uint64_t digit = 0;
    if (t <= c.lev) {
      const int s = c.lev - t;
      for (int d = 0; d < m.dim; ++d) digit |= (uint64_t)((c.x[d] >> s) & 1) << d;
    }
    key = (key << m.dim) | digit;
  }
  return key;
}

// level-`lev` cells whose closure holds position p (up to 2 per axis), active ones only; the
// smallest active index, or -1
int first_containing(const AmrMesh& m, int lev, const std::array<long long, 3>& p) {
  const long long W = (long long)m.k << (m.maxlev - lev);
  long long cand[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  int ncand[3] = {1, 1, 1};
  for (int d = 0; d < m.dim; ++d) {
    const long long q = p[d] / W, r = p[d] % W;
    ncand[d] = 0;
    const long long opts[2] = {q - 1, q};
    for (int o = r == 0 ? 0 : 1; o < 2; ++o) {
      long long y = opts[o];
      if (!wrap(m, d, lev, y)) continue;
      bool dup = false;
      for (int e = 0; e < ncand[d]; ++e) dup |= cand[d][e] == y;
      if (!dup) cand[d][ncand[d]++] = y;
    }
    if (ncand[d] == 0) return -1;
  }
  int best = -1;
  for (int a = 0; a < ncand[0]; ++a)
    for (int b = 0; b < ncand[1]; ++b)
      for (int e = 0; e < ncand[2]; ++e) {
        const int i = m.find(lev, cand[0][a], cand[1][b], cand[2][e]);
        if (i >= 0 && (best < 0 || i < best)) best = i;
      }
  return best;
}

}  // namespace

uint64_t AmrMesh::cell_key(int lev, long long x, long long y, long long z) const {
  return ((uint64_t)lev << (3 * KEY_BITS)) | ((uint64_t)z << (2 * KEY_BITS)) | ((uint64_t)y << KEY_BITS) | (uint64_t)x;
}

uint64_t AmrMesh::pos_key(const std::array<long long, 3>& p) const {
  return ((uint64_t)p[2] << (2 * POS_BITS)) | ((uint64_t)p[1] << POS_BITS) | (uint64_t)p[0];
}

int AmrMesh::find(int lev, long long x, long long y, long long z) const {
  auto it = index.find(cell_key(lev, x, y, z));
  return it == index.end() ? -1 : it->second;
}

void amr_set_cells(AmrMesh& m, std::vector<AmrCell> cells) {
  struct Item {
    long long coarse;
    uint64_t path;
    AmrCell c;
  };
  std::vector<Item> items;
  items.reserve(cells.size());
  for (auto& c : cells) {
    long long q[3] = {0, 0, 0};
    for (int d = 0; d < m.dim; ++d) q[d] = (long long)c.x[d] >> c.lev;
    const long long coarse = q[0] + (long long)m.sub[0] * (q[1] + (long long)m.sub[1] * q[2]);
    items.push_back({coarse, path_key(m, c), c});
  }
  std::sort(items.begin(), items.end(), [](const Item& a, const Item& b) {
    return a.coarse != b.coarse ? a.coarse < b.coarse : a.path < b.path;
  });
  m.cells.resize(items.size());
  m.index.clear();
  m.index.reserve(items.size() * 2);
  for (size_t i = 0; i < items.size(); ++i) {
    m.cells[i] = items[i].c;
    const AmrCell& c = m.cells[i];
    m.index[m.cell_key(c.lev, c.x[0], c.x[1], c.x[2])] = (int)i;
  }
}

bool amr_init_uniform(AmrMesh& m, int dim, int degree, const int* subdivisions, const int* periodic, int level,
                      int max_level, std::string& err) {
  if (dim < 2 || dim > 3 || degree < 1 || degree > 2) {
    err = "adaptive meshes need dim 2 or 3 and degree 1 or 2";
    return false;
  }
  if (level < 0 || max_level < level) {
    err = "adaptive meshes need 0 <= global refinement <= max refinement";
    return false;
  }
  m.dim = dim;
  m.k = degree;
  m.n = degree + 1;
  m.nq = dim == 2 ? m.n * m.n : m.n * m.n * m.n;
  m.maxlev = max_level;
  for (int d = 0; d < 3; ++d) {
    m.sub[d] = d < dim ? subdivisions[d] : 1;
    m.periodic[d] = d < dim ? (periodic[d] != 0) : 0;
    if (d < dim && (((long long)m.sub[d] << max_level) >= (1LL << KEY_BITS) ||
                    (((long long)m.sub[d] * degree) << max_level) >= (1LL << POS_BITS))) {
      err = "adaptive mesh too fine for the position encoding (subdivisions * 2^max refinement too large)";
      return false;
    }
    m.E[d] = d < dim ? ((long long)m.sub[d] * degree) << max_level : 1;
  }
  std::vector<AmrCell> cells;
  const long long nx = (long long)m.sub[0] << level, ny = (long long)m.sub[1] << level,
                  nz = dim == 3 ? (long long)m.sub[2] << level : 1;
  cells.reserve((size_t)(nx * ny * nz));
  for (long long z = 0; z < nz; ++z)
    for (long long y = 0; y < ny; ++y)
      for (long long x = 0; x < nx; ++x) cells.push_back({level, {(int)x, (int)y, (int)z}});
  amr_set_cells(m, std::move(cells));
  return true;
}

void amr_build(AmrMesh& m) {
  const int nq = m.nq, n = m.n, k = m.k;
  const long long nc = m.ncells();
  m.cell_dofs.assign((size_t)nc * nq, 0);
  m.pos.clear();
  m.node_of.clear();
  m.node_of.reserve((size_t)nc * nq);
  std::vector<int> minlev;
  for (long long c = 0; c < nc; ++c) {
    const AmrCell& C = m.cells[c];
    const int s = m.maxlev - C.lev;
    for (int l = 0; l < nq; ++l) {
      const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
      std::array<long long, 3> p{0, 0, 0};
      for (int d = 0; d < m.dim; ++d) {
        long long q = ((long long)C.x[d] * k + idx[d]) << s;
        if (m.periodic[d] && q == m.E[d]) q = 0;
        p[d] = q;
      }
      const uint64_t key = m.pos_key(p);
      auto it = m.node_of.find(key);
      int dof;
      if (it == m.node_of.end()) {
        dof = (int)m.pos.size();
        m.node_of.emplace(key, dof);
        m.pos.push_back(p);
        minlev.push_back(C.lev);
      } else {
        dof = it->second;
        minlev[dof] = std::min(minlev[dof], C.lev);
      }
      m.cell_dofs[(size_t)c * nq + l] = dof;
    }
  }
  m.N = (long long)m.pos.size();
  // hanging lines before closure: each DoF against the active cells one level coarser than its
  // coarsest incident cell (2:1 balance leaves no other candidates); the first in cell order
  std::vector<std::vector<std::pair<int, double>>> raw(m.N);
  for (long long p = 0; p < m.N; ++p) {
    const int lev = minlev[p] - 1;
    if (lev < 0) continue;
    const int best = first_containing(m, lev, m.pos[p]);
    if (best < 0) continue;
    const AmrCell& C = m.cells[best];
    long long off[3] = {0, 0, 0};
    if (!local_offset(m, C.lev, C.x, m.pos[p], off)) continue;
    const double W = (double)((long long)k << (m.maxlev - lev));
    for (int l = 0; l < nq; ++l) {
      const int idx[3] = {l % n, (l / n) % n, l / (n * n)};
      double wl = 1.0;
      for (int d = 0; d < m.dim; ++d) wl *= lagrange_exact(k, idx[d], (double)off[d] / W);
      if (wl != 0.0) raw[p].push_back({m.cell_dofs[(size_t)best * nq + l], wl});
    }
  }
  // closure over hanging masters (AffineConstraints::close)
  std::vector<std::vector<std::pair<int, double>>> closed(m.N);
  std::vector<char> done(m.N, 0);
  std::function<const std::vector<std::pair<int, double>>&(int)> resolve;
  resolve = [&](int p) -> const std::vector<std::pair<int, double>>& {
    if (done[p]) return closed[p];
    std::vector<std::pair<int, double>> out;
    for (auto& e : raw[p]) {
      if (raw[e.first].empty()) {
        out.push_back(e);
      } else {
        for (auto& f : resolve(e.first)) out.push_back({f.first, e.second * f.second});
      }
    }
    std::sort(out.begin(), out.end());
    std::vector<std::pair<int, double>> merged;
    for (auto& e : out) {
      if (!merged.empty() && merged.back().first == e.first) merged.back().second += e.second;
      else merged.push_back(e);
    }
    closed[p] = std::move(merged);
    done[p] = 1;
    return closed[p];
  };
  m.hang_row.assign(m.N, -1);
  m.h_dof.clear();
  m.h_ptr.assign(1, 0);
  m.h_idx.clear();
  m.h_w.clear();
  for (long long p = 0; p < m.N; ++p) {
    if (raw[p].empty()) continue;
    const auto& line = resolve((int)p);
    m.hang_row[p] = (int)m.h_dof.size();
    m.h_dof.push_back((int)p);
    for (auto& e : line) {
      m.h_idx.push_back(e.first);
      m.h_w.push_back(e.second);
    }
    m.h_ptr.push_back((int)m.h_idx.size());
  }
}

void amr_smooth(const AmrMesh& m, std::vector<signed char>& flag, int max_level) {
  const int nc = (int)m.ncells();
  const int nchild = 1 << m.dim;
  std::vector<std::vector<int>> touch(nc);
  for (int c = 0; c < nc; ++c) touching(m, c, touch[c]);
  std::vector<std::vector<std::vector<int>>> faces(nc, std::vector<std::vector<int>>(2 * m.dim));
  for (int c = 0; c < nc; ++c)
    for (int d = 0; d < m.dim; ++d)
      for (int s = 0; s < 2; ++s) touching(m, c, faces[c][2 * d + s], d, s);
  auto parent = [&](int c) {
    const AmrCell& C = m.cells[c];
    return m.cell_key(C.lev - 1, C.x[0] >> 1, C.x[1] >> 1, C.x[2] >> 1);
  };
  auto target = [&](int c) { return m.cells[c].lev + (flag[c] == 1) - (flag[c] == -1); };
  for (;;) {
    bool changed = false;
    std::unordered_map<uint64_t, int> fam;
    for (int c = 0; c < nc; ++c)
      if (flag[c] == -1) fam[parent(c)]++;
    for (int c = 0; c < nc; ++c)
      if (flag[c] == -1 && fam[parent(c)] != nchild) {
        flag[c] = 0;
        changed = true;
      }
    for (int a = 0; a < nc; ++a) {
      const int ta = target(a);
      for (int b : touch[a]) {
        if (ta <= target(b) + 1) continue;
        const signed char nf = flag[b] == -1 ? 0 : 1;
        if (nf != flag[b]) {
          flag[b] = nf;
          changed = true;
        }
      }
    }
    for (int a = 0; a < nc; ++a) {
      if (flag[a] == 1) continue;
      int refined = 0, unrefined = 0;
      for (int f = 0; f < 2 * m.dim; ++f) {
        const auto& nb = faces[a][f];
        if (nb.empty()) continue;  // domain boundary
        bool fine = false;
        for (int b : nb)
          fine |= m.cells[b].lev > m.cells[a].lev || (m.cells[b].lev == m.cells[a].lev && flag[b] == 1);
        if (fine) ++refined;
        else ++unrefined;
      }
      if (refined > unrefined && m.cells[a].lev < max_level) {
        flag[a] = 1;
        changed = true;
      }
    }
    if (!changed) break;
  }
}

std::vector<AmrCell> amr_refine(const AmrMesh& m, const std::vector<signed char>& flag) {
  std::vector<AmrCell> out;
  out.reserve(m.cells.size() * 2);
  std::unordered_set<uint64_t> parents;
  for (size_t c = 0; c < m.cells.size(); ++c) {
    const AmrCell& C = m.cells[c];
    if (flag[c] == 1) {
      for (int ch = 0; ch < (1 << m.dim); ++ch)
        out.push_back({C.lev + 1,
                       {2 * C.x[0] + (ch & 1), 2 * C.x[1] + ((ch >> 1) & 1), m.dim == 3 ? 2 * C.x[2] + ((ch >> 2) & 1) : 0}});
    } else if (flag[c] == -1) {
      const uint64_t pk = m.cell_key(C.lev - 1, C.x[0] >> 1, C.x[1] >> 1, C.x[2] >> 1);
      if (parents.insert(pk).second) out.push_back({C.lev - 1, {C.x[0] >> 1, C.x[1] >> 1, C.x[2] >> 1}});
    } else {
      out.push_back(C);
    }
  }
  return out;
}

void amr_transfer_plan(const AmrMesh& old, const AmrMesh& m, std::vector<int>& ptr, std::vector<int>& idx,
                       std::vector<double>& w) {
  ptr.assign(1, 0);
  idx.clear();
  w.clear();
  const int nq = m.nq, n = m.n;
  for (long long p = 0; p < m.N; ++p) {
    auto it = old.node_of.find(old.pos_key(m.pos[p]));
    if (it != old.node_of.end()) {
      idx.push_back(it->second);
      w.push_back(1.0);
      ptr.push_back((int)idx.size());
      continue;
    }
    // first old cell (in old order) whose closure holds the new node
    int best = -1;
    for (int lev = 0; lev <= old.maxlev; ++lev) {
      const int i = first_containing(old, lev, m.pos[p]);
      if (i >= 0 && (best < 0 || i < best)) best = i;
    }
    if (best >= 0) {
      const AmrCell& C = old.cells[best];
      long long off[3] = {0, 0, 0};
      local_offset(old, C.lev, C.x, m.pos[p], off);
      const double W = (double)((long long)old.k << (old.maxlev - C.lev));
      for (int l = 0; l < nq; ++l) {
        const int id[3] = {l % n, (l / n) % n, l / (n * n)};
        double wl = 1.0;
        for (int d = 0; d < m.dim; ++d) wl *= lagrange_exact(m.k, id[d], (double)off[d] / W);
        if (wl != 0.0) {
          idx.push_back(old.cell_dofs[(size_t)best * nq + l]);
          w.push_back(wl);
        }
      }
    }
    ptr.push_back((int)idx.size());
  }
}

void amr_point(const AmrMesh& m, const double* lower, const double* size, long long p, double* x) {
  for (int d = 0; d < 3; ++d)
    x[d] = d < m.dim ? lower[d] + size[d] * ((double)m.pos[p][d] / (double)m.E[d]) : 0.0;
}

}  // namespace ppf
