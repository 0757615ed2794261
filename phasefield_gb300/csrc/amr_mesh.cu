// Host-side adaptive mesh (forest of quadtrees / octrees): see amr_mesh.h.
#include "amr_mesh.h"

#include <algorithm>
#include <functional>
#include <thread>
#include <unordered_map>
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
  // a balanced mesh has the region's parent or its children active: try those first
  if (lev > 0) {
    const int a = m.find(lev - 1, y0 >> 1, y1 >> 1, y2 >> 1);
    if (a >= 0) {
      out.push_back(a);
      return;
    }
  }
  if (lev < m.maxlev) {
    const size_t before = out.size();
    bool all = true;
    for (int ch = 0; ch < (1 << m.dim) && all; ++ch) {
      long long c[3] = {0, 0, 0};
      bool ok = true;
      for (int d = 0; d < m.dim; ++d) {
        const int b = (ch >> d) & 1;
        if (dir[d] > 0 && b != 1) ok = false;
        if (dir[d] < 0 && b != 0) ok = false;
        c[d] = 2 * (d == 0 ? y0 : d == 1 ? y1 : y2) + b;
      }
      if (!ok) continue;
      const int j = m.find(lev + 1, c[0], c[1], c[2]);
      if (j >= 0) out.push_back(j);
      else all = false;
    }
    if (all && out.size() > before) return;
    out.resize(before);
  }
  for (int l = lev - 2; l >= 0; --l) {
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

// Neighbours of cell c: the active cells touching it (sharing at least a vertex), appended to
// `touch` without c itself or repeats, and per face (axis, side) whether a neighbour exists and
// whether one of them is finer than c or flagged for refinement at c's level (`fine` per face
// is filled by the caller from `faces`, the face neighbours appended per face).
void neighbours(const AmrMesh& m, int c, std::vector<int>& touch, std::vector<int> faces[6], std::vector<int>& scratch) {
  const AmrCell& C = m.cells[c];
  const int nd = m.dim;
  int total = 1;
  for (int d = 0; d < nd; ++d) total *= 3;
  const size_t t0 = touch.size();
  for (int t = 0; t < total; ++t) {
    int delta[3] = {0, 0, 0};
    int r = t, nz = 0, axis = -1;
    for (int d = 0; d < nd; ++d) {
      delta[d] = r % 3 - 1;
      r /= 3;
      if (delta[d] != 0) {
        ++nz;
        axis = d;
      }
    }
    if (nz == 0) continue;
    long long y[3] = {0, 0, 0};
    bool inside = true;
    for (int d = 0; d < nd; ++d) {
      y[d] = (long long)C.x[d] + delta[d];
      inside &= wrap(m, d, C.lev, y[d]);
    }
    if (!inside) continue;
    const int back[3] = {-delta[0], -delta[1], -delta[2]};
    scratch.clear();
    covering(m, C.lev, y[0], y[1], y[2], back, scratch);
    for (int b : scratch) {
      if (b == c) continue;
      touch.push_back(b);
      if (nz == 1) faces[2 * axis + (delta[axis] > 0)].push_back(b);
    }
  }
  std::sort(touch.begin() + t0, touch.end());
  touch.erase(std::unique(touch.begin() + t0, touch.end()), touch.end());
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

// fn(begin, end, chunk) over [0, n) in contiguous chunks on host threads (one chunk for small n)
template <class Fn>
int parallel_chunks(long long n, Fn fn) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const int nchunk = (int)std::min<long long>(hw, std::max<long long>(1, n / 2048));
  std::vector<std::thread> pool;
  for (int k = 1; k < nchunk; ++k) pool.emplace_back(fn, n * k / nchunk, n * (k + 1) / nchunk, k);
  fn(0, n / nchunk, 0);
  for (auto& t : pool) t.join();
  return nchunk;
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

static inline uint64_t mix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

void KeyTable::reset(size_t expected) {
  size_t cap = 16;
  while (cap < 2 * expected + 2) cap <<= 1;
  keys_.assign(cap, EMPTY);
  vals_.assign(cap, -1);
  mask_ = cap - 1;
  count_ = 0;
}

int KeyTable::find(uint64_t key) const {
  if (keys_.empty()) return -1;
  for (uint64_t i = mix64(key) & mask_;; i = (i + 1) & mask_) {
    if (keys_[i] == key) return vals_[i];
    if (keys_[i] == EMPTY) return -1;
  }
}

void KeyTable::grow() {
  std::vector<uint64_t> k = std::move(keys_);
  std::vector<int> v = std::move(vals_);
  reset(k.size());
  bool ins;
  for (size_t i = 0; i < k.size(); ++i)
    if (k[i] != EMPTY) insert(k[i], v[i], ins);
}

int KeyTable::insert(uint64_t key, int value, bool& inserted) {
  if (keys_.empty() || 2 * (count_ + 1) > keys_.size()) grow();
  for (uint64_t i = mix64(key) & mask_;; i = (i + 1) & mask_) {
    if (keys_[i] == key) {
      inserted = false;
      return vals_[i];
    }
    if (keys_[i] == EMPTY) {
      keys_[i] = key;
      vals_[i] = value;
      ++count_;
      inserted = true;
      return value;
    }
  }
}

uint64_t AmrMesh::cell_key(int lev, long long x, long long y, long long z) const {
  return ((uint64_t)lev << (3 * KEY_BITS)) | ((uint64_t)z << (2 * KEY_BITS)) | ((uint64_t)y << KEY_BITS) | (uint64_t)x;
}

uint64_t AmrMesh::pos_key(const std::array<long long, 3>& p) const {
  return ((uint64_t)p[2] << (2 * POS_BITS)) | ((uint64_t)p[1] << POS_BITS) | (uint64_t)p[0];
}

int AmrMesh::find(int lev, long long x, long long y, long long z) const {
  return index.find(cell_key(lev, x, y, z));
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
  // refining in place keeps tree order (children replace their parent in child order, a
  // coarsened family's parent takes its first child's place): sort only when that fails
  auto before = [](const Item& a, const Item& b) { return a.coarse != b.coarse ? a.coarse < b.coarse : a.path < b.path; };
  if (!std::is_sorted(items.begin(), items.end(), before)) std::sort(items.begin(), items.end(), before);
  m.cells.resize(items.size());
  m.index.reset(items.size());
  for (size_t i = 0; i < items.size(); ++i) {
    m.cells[i] = items[i].c;
    const AmrCell& c = m.cells[i];
    bool ins;
    m.index.insert(m.cell_key(c.lev, c.x[0], c.x[1], c.x[2]), (int)i, ins);
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
  m.node_of.reset((size_t)nc * (m.dim == 2 ? 2 : 3));
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
      bool fresh;
      const int dof = m.node_of.insert(key, (int)m.pos.size(), fresh);
      if (fresh) {
        m.pos.push_back(p);
        minlev.push_back(C.lev);
      } else {
        minlev[dof] = std::min(minlev[dof], C.lev);
      }
      m.cell_dofs[(size_t)c * nq + l] = dof;
    }
  }
  m.N = (long long)m.pos.size();
  // hanging lines before closure: each DoF against the active cells one level coarser than its
  // coarsest incident cell (2:1 balance leaves no other candidates); the first in cell order
  std::vector<std::vector<std::pair<int, double>>> raw(m.N);
  parallel_chunks(m.N, [&](long long p0, long long p1, int) {
    for (long long p = p0; p < p1; ++p) {
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
  });
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
  const int nf = 2 * m.dim;
  // neighbour lists, flat: touching cells and face neighbours per (cell, face); built by
  // independent chunks of cells on host threads, then joined in cell order
  std::vector<int> t_ptr(nc + 1, 0), touch, f_ptr((size_t)nc * nf + 1, 0), fnb;
  {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int nchunk = (int)std::min<long long>(hw, std::max(1, nc / 2048));
    struct Part {
      std::vector<int> touch, tcount, fnb, fcount;
    };
    std::vector<Part> parts(nchunk);
    auto work = [&](int k) {
      Part& P = parts[k];
      const int c0 = (int)((long long)nc * k / nchunk), c1 = (int)((long long)nc * (k + 1) / nchunk);
      std::vector<int> faces[6], scratch;
      for (int c = c0; c < c1; ++c) {
        for (int f = 0; f < nf; ++f) faces[f].clear();
        const size_t t0 = P.touch.size();
        neighbours(m, c, P.touch, faces, scratch);
        P.tcount.push_back((int)(P.touch.size() - t0));
        for (int f = 0; f < nf; ++f) {
          std::sort(faces[f].begin(), faces[f].end());
          faces[f].erase(std::unique(faces[f].begin(), faces[f].end()), faces[f].end());
          P.fnb.insert(P.fnb.end(), faces[f].begin(), faces[f].end());
          P.fcount.push_back((int)faces[f].size());
        }
      }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < nchunk; ++k) pool.emplace_back(work, k);
    work(0);
    for (auto& t : pool) t.join();
    int c = 0;
    size_t cf = 0;
    for (const Part& P : parts) {
      touch.insert(touch.end(), P.touch.begin(), P.touch.end());
      fnb.insert(fnb.end(), P.fnb.begin(), P.fnb.end());
      for (int n : P.tcount) {
        t_ptr[c + 1] = t_ptr[c] + n;
        ++c;
      }
      for (int n : P.fcount) {
        f_ptr[cf + 1] = f_ptr[cf] + n;
        ++cf;
      }
    }
  }
  // in tree order a family of active siblings is the 2^dim consecutive cells starting at the
  // first child: complete when all of them are active at the child's level under one parent
  auto complete_family = [&](int c) {
    const AmrCell& C = m.cells[c];
    int ci = 0;
    for (int d = 0; d < m.dim; ++d) ci |= (C.x[d] & 1) << d;
    const int s = c - ci;
    if (s < 0 || s + nchild > nc) return false;
    for (int j = 0; j < nchild; ++j) {
      const AmrCell& S = m.cells[s + j];
      if (S.lev != C.lev || flag[s + j] != -1) return false;
      for (int d = 0; d < m.dim; ++d)
        if ((S.x[d] >> 1) != (C.x[d] >> 1) || (S.x[d] & 1) != ((j >> d) & 1)) return false;
    }
    return true;
  };
  auto target = [&](int c) { return m.cells[c].lev + (flag[c] == 1) - (flag[c] == -1); };
  std::vector<char> clear;
  for (;;) {
    bool changed = false;
    clear.assign(nc, 0);
    for (int c = 0; c < nc; ++c)
      if (flag[c] == -1 && !complete_family(c)) clear[c] = 1;
    for (int c = 0; c < nc; ++c)
      if (clear[c]) {
        flag[c] = 0;
        changed = true;
      }
    for (int a = 0; a < nc; ++a) {
      const int ta = target(a);
      for (int e = t_ptr[a]; e < t_ptr[a + 1]; ++e) {
        const int b = touch[e];
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
      for (int f = 0; f < nf; ++f) {
        const int e0 = f_ptr[(size_t)a * nf + f], e1 = f_ptr[(size_t)a * nf + f + 1];
        if (e0 == e1) continue;  // domain boundary
        bool fine = false;
        for (int e = e0; e < e1; ++e) {
          const int b = fnb[e];
          fine |= m.cells[b].lev > m.cells[a].lev || (m.cells[b].lev == m.cells[a].lev && flag[b] == 1);
        }
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
  const int nq = m.nq, n = m.n;
  // rows built per chunk of new DoFs on host threads, then joined in DoF order
  struct Part {
    std::vector<int> cnt, idx;
    std::vector<double> w;
  };
  std::vector<Part> parts(16);
  const int nchunk = parallel_chunks(m.N, [&](long long p0, long long p1, int k) {
    Part& P = parts[k];
    for (long long p = p0; p < p1; ++p) {
      const size_t e0 = P.idx.size();
      const int same = old.node_of.find(old.pos_key(m.pos[p]));
      if (same >= 0) {
        P.idx.push_back(same);
        P.w.push_back(1.0);
        P.cnt.push_back(1);
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
            P.idx.push_back(old.cell_dofs[(size_t)best * nq + l]);
            P.w.push_back(wl);
          }
        }
      }
      P.cnt.push_back((int)(P.idx.size() - e0));
    }
  });
  ptr.assign(1, 0);
  ptr.reserve(m.N + 1);
  idx.clear();
  w.clear();
  for (int k = 0; k < nchunk; ++k) {
    const Part& P = parts[k];
    for (int c : P.cnt) ptr.push_back(ptr.back() + c);
    idx.insert(idx.end(), P.idx.begin(), P.idx.end());
    w.insert(w.end(), P.w.begin(), P.w.end());
  }
}

void amr_point(const AmrMesh& m, const double* lower, const double* size, long long p, double* x) {
  for (int d = 0; d < 3; ++d)
    x[d] = d < m.dim ? lower[d] + size[d] * ((double)m.pos[p][d] / (double)m.E[d]) : 0.0;
}

}  // namespace ppf
