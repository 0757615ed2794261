// Test infrastructure: a C interface to the engine's host-side adaptive mesh
// (phasefield_gb300/csrc/amr_mesh.cu) for tests/test_amr_mesh_host.py, which compiles it with
// g++ together with amr_mesh.cu (plain C++, no CUDA) and compares it with the oracle on the CPU.
#include <cstring>
#include <string>
#include <vector>

#include "amr_mesh.h"

using namespace ppf;

extern "C" {

void* shim_uniform(int dim, int degree, const int* sub, const int* per, int level, int max_level) {
  auto* m = new AmrMesh();
  std::string err;
  if (!amr_init_uniform(*m, dim, degree, sub, per, level, max_level, err)) {
    delete m;
    return nullptr;
  }
  amr_build(*m);
  return m;
}

void shim_free(void* m) { delete static_cast<AmrMesh*>(m); }

long long shim_ncells(void* m) { return static_cast<AmrMesh*>(m)->ncells(); }
long long shim_ndofs(void* m) { return static_cast<AmrMesh*>(m)->N; }

void shim_cells(void* p, int* out) {
  const AmrMesh& m = *static_cast<AmrMesh*>(p);
  for (long long c = 0; c < m.ncells(); ++c) {
    out[4 * c] = m.cells[c].lev;
    for (int d = 0; d < 3; ++d) out[4 * c + 1 + d] = m.cells[c].x[d];
  }
}

void shim_cell_dofs(void* p, int* out) {
  const AmrMesh& m = *static_cast<AmrMesh*>(p);
  std::memcpy(out, m.cell_dofs.data(), sizeof(int) * m.cell_dofs.size());
}

long long shim_hanging(void* p, int* count, int* master, double* weight) {
  const AmrMesh& m = *static_cast<AmrMesh*>(p);
  if (count)
    for (long long i = 0; i < m.N; ++i) count[i] = m.hang_row[i] < 0 ? 0 : m.h_ptr[m.hang_row[i] + 1] - m.h_ptr[m.hang_row[i]];
  if (master) std::memcpy(master, m.h_idx.data(), sizeof(int) * m.h_idx.size());
  if (weight) std::memcpy(weight, m.h_w.data(), sizeof(double) * m.h_w.size());
  return (long long)m.h_idx.size();
}

// smooths the marks in place and returns the refined/coarsened mesh (numbered, with its lines)
void* shim_refine(void* p, signed char* flags, int max_level) {
  const AmrMesh& m = *static_cast<AmrMesh*>(p);
  std::vector<signed char> f(flags, flags + m.ncells());
  amr_smooth(m, f, max_level);
  std::memcpy(flags, f.data(), f.size());
  auto* nm = new AmrMesh();
  nm->dim = m.dim;
  nm->k = m.k;
  nm->n = m.n;
  nm->nq = m.nq;
  nm->maxlev = m.maxlev;
  for (int d = 0; d < 3; ++d) {
    nm->sub[d] = m.sub[d];
    nm->periodic[d] = m.periodic[d];
    nm->E[d] = m.E[d];
  }
  amr_set_cells(*nm, amr_refine(m, f));
  amr_build(*nm);
  return nm;
}

// transfer plan old -> new; returns the entry count (outputs may be null to size them)
long long shim_transfer(void* old, void* nm, int* ptr, int* idx, double* w) {
  std::vector<int> p, i;
  std::vector<double> v;
  amr_transfer_plan(*static_cast<AmrMesh*>(old), *static_cast<AmrMesh*>(nm), p, i, v);
  if (ptr) std::memcpy(ptr, p.data(), sizeof(int) * p.size());
  if (idx) std::memcpy(idx, i.data(), sizeof(int) * i.size());
  if (w) std::memcpy(w, v.data(), sizeof(double) * v.size());
  return (long long)i.size();
}

}  // extern "C"
