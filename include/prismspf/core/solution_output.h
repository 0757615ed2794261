// VTU output of the solution fields (reference: include/prismspf/core/solution_output.h:45-160,
// deal.II DataOut::build_patches + write_vtu).
//
// Like build_patches(n_subdivisions), every cell becomes a patch of n_subdivisions^dim
// sub-cells whose (n_subdivisions+1)^dim points sit at equidistant positions in the cell;
// the finite-element solution (degree-k Lagrange on Gauss-Lobatto nodes) is evaluated there.
// Scalar fields are written as one component, vector fields as three (zero-padded in 2-D),
// under the field's name. TIME and CYCLE are stored as field data. Data are raw appended
// binary (UInt64 block headers, Float64 values, Int64 connectivity).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <prismspf/config.h>

PRISMS_PF_BEGIN_NAMESPACE

namespace output {

// Gauss-Lobatto nodes on [0, 1] for degree k (1..4)
inline std::vector<double> gauss_lobatto_unit(int k) {
  switch (k) {
    case 1: return {0.0, 1.0};
    case 2: return {0.0, 0.5, 1.0};
    case 3: {
      const double a = 0.5 / std::sqrt(5.0);
      return {0.0, 0.5 - a, 0.5 + a, 1.0};
    }
    case 4: {
      const double a = 0.5 * std::sqrt(3.0 / 7.0);
      return {0.0, 0.5 - a, 0.5, 0.5 + a, 1.0};
    }
    default: throw std::invalid_argument("degree must be 1..4");
  }
}

// 1-D Lagrange basis on `nodes` evaluated at `x`: L[p][j] = l_j(x_p)
inline std::vector<std::vector<double>> lagrange_matrix(const std::vector<double>& nodes, const std::vector<double>& x) {
  std::vector<std::vector<double>> L(x.size(), std::vector<double>(nodes.size(), 1.0));
  for (size_t p = 0; p < x.size(); ++p)
    for (size_t j = 0; j < nodes.size(); ++j)
      for (size_t m = 0; m < nodes.size(); ++m)
        if (m != j) L[p][j] *= (x[p] - nodes[m]) / (nodes[j] - nodes[m]);
  return L;
}

struct Lattice {
  int dim = 2, degree = 1;
  int nc[3] = {1, 1, 1};   // cells per axis
  int nn[3] = {1, 1, 1};   // nodes per axis
  double lower[3] = {0, 0, 0};
  double h[3] = {1, 1, 1};
  long long N = 0;
};

struct OutputField {
  std::string name;
  int ncomp = 1;                   // 1 or dim
  const double* values = nullptr;  // lattice (or cell-list DoF) order, component-major
};

// The active cells of an adaptive mesh: level and integer coordinates at that level per cell
// (4 ints each), the DoF index of each cell's (degree+1)^dim lexicographic nodes, the DoF
// count per component, and the coarse mesh (subdivisions, size) the levels refine.
struct CellList {
  long long ncells = 0;
  const int* cells = nullptr;
  const int* cell_dofs = nullptr;
  long long N = 0;
  int subdivisions[3] = {1, 1, 1};
  double size[3] = {1, 1, 1};
};

class VTUWriter {
 public:
  VTUWriter(const Lattice& L, unsigned int n_subdivisions) : lat(L), ns(n_subdivisions ? n_subdivisions : L.degree) {
    init();
  }
  // cells of an adaptive mesh; `L` gives dim, degree and the lower corner
  VTUWriter(const Lattice& L, const CellList& C, unsigned int n_subdivisions)
      : lat(L), cl(&C), ns(n_subdivisions ? n_subdivisions : L.degree) {
    lat.N = C.N;
    init();
  }

  void init() {
    nodes = gauss_lobatto_unit(lat.degree);
    std::vector<double> xe(ns + 1);
    for (unsigned i = 0; i <= ns; ++i) xe[i] = double(i) / ns;
    I = lagrange_matrix(nodes, xe);
  }

  void write(const std::string& filename, const std::vector<OutputField>& fields, double time, unsigned int cycle) const {
    const int dim = lat.dim, k = lat.degree;
    const int np1 = ns + 1;
    const long long ncells = cl ? cl->ncells : (long long)lat.nc[0] * lat.nc[1] * lat.nc[2];
    const long long ppc = dim == 2 ? (long long)np1 * np1 : (long long)np1 * np1 * np1;  // points per cell
    const long long scc = dim == 2 ? (long long)ns * ns : (long long)ns * ns * ns;        // sub-cells per cell
    const long long npts = ncells * ppc, nsub = ncells * scc;
    std::vector<double> pts(3 * npts, 0.0);
    std::vector<std::vector<double>> data(fields.size());
    for (size_t f = 0; f < fields.size(); ++f) data[f].assign(3 * npts * (fields[f].ncomp > 1) + npts * (fields[f].ncomp == 1), 0.0);
    const int n = k + 1;
    std::vector<double> cellv(n * n * (dim == 3 ? n : 1));
    long long p = 0;
    const int ncn = dim == 3 ? n * n * n : n * n;
    for (long long c = 0; c < ncells; ++c) {
      int cx, cy, cz;
      double hc[3] = {lat.h[0], lat.h[1], lat.h[2]};
      if (cl) {
        const int lev = cl->cells[4 * c];
        cx = cl->cells[4 * c + 1];
        cy = cl->cells[4 * c + 2];
        cz = cl->cells[4 * c + 3];
        for (int d = 0; d < dim; ++d) hc[d] = cl->size[d] / (int)((long long)cl->subdivisions[d] << lev);
      } else {
        cx = (int)(c % lat.nc[0]);
        cy = (int)((c / lat.nc[0]) % lat.nc[1]);
        cz = (int)(c / ((long long)lat.nc[0] * lat.nc[1]));
      }
      for (int pz = 0; pz < (dim == 3 ? np1 : 1); ++pz)
        for (int py = 0; py < np1; ++py)
          for (int px = 0; px < np1; ++px) {
            const long long q = p + (dim == 3 ? ((long long)pz * np1 + py) * np1 + px : (long long)py * np1 + px);
            pts[3 * q + 0] = lat.lower[0] + hc[0] * (cx + double(px) / ns);
            pts[3 * q + 1] = lat.lower[1] + hc[1] * (cy + double(py) / ns);
            pts[3 * q + 2] = dim == 3 ? lat.lower[2] + hc[2] * (cz + double(pz) / ns) : 0.0;
          }
      for (size_t f = 0; f < fields.size(); ++f) {
        const OutputField& F = fields[f];
        for (int comp = 0; comp < F.ncomp; ++comp) {
          const double* u = F.values + (long long)comp * lat.N;
          for (int c3 = 0; c3 < (dim == 3 ? n : 1); ++c3)
            for (int b = 0; b < n; ++b)
              for (int a = 0; a < n; ++a)
                cellv[(c3 * n + b) * n + a] =
                    cl ? u[cl->cell_dofs[c * ncn + (c3 * n + b) * n + a]]
                       : u[((long long)(k * cz + c3) * lat.nn[1] + (k * cy + b)) * lat.nn[0] + (k * cx + a)];
          for (int pz = 0; pz < (dim == 3 ? np1 : 1); ++pz)
            for (int py = 0; py < np1; ++py)
              for (int px = 0; px < np1; ++px) {
                double s = 0.0;
                for (int c3 = 0; c3 < (dim == 3 ? n : 1); ++c3) {
                  const double wz = dim == 3 ? I[pz][c3] : 1.0;
                  for (int b = 0; b < n; ++b)
                    for (int a = 0; a < n; ++a) s += wz * I[py][b] * I[px][a] * cellv[(c3 * n + b) * n + a];
                }
                const long long q = p + (dim == 3 ? ((long long)pz * np1 + py) * np1 + px : (long long)py * np1 + px);
                if (F.ncomp == 1) data[f][q] = s;
                else data[f][3 * q + comp] = s;
              }
        }
      }
      p += ppc;
    }
    // connectivity of the sub-cells (VTK vertex order)
    const int nvert = dim == 2 ? 4 : 8;
    std::vector<int64_t> conn(nsub * nvert), offs(nsub);
    std::vector<uint8_t> types(nsub, dim == 2 ? 9 : 12);
    long long s = 0;
    for (long long c = 0; c < ncells; ++c) {
      const long long base = c * ppc;
      auto id = [&](int x, int y, int z) { return base + (dim == 3 ? ((long long)z * np1 + y) * np1 + x : (long long)y * np1 + x); };
      for (unsigned z = 0; z < (dim == 3 ? ns : 1); ++z)
        for (unsigned y = 0; y < ns; ++y)
          for (unsigned x = 0; x < ns; ++x) {
            int64_t* v = &conn[s * nvert];
            v[0] = id(x, y, z);
            v[1] = id(x + 1, y, z);
            v[2] = id(x + 1, y + 1, z);
            v[3] = id(x, y + 1, z);
            if (dim == 3) {
              v[4] = id(x, y, z + 1);
              v[5] = id(x + 1, y, z + 1);
              v[6] = id(x + 1, y + 1, z + 1);
              v[7] = id(x, y + 1, z + 1);
            }
            offs[s] = (s + 1) * nvert;
            ++s;
          }
    }
    const std::filesystem::path path(filename);
    if (path.has_parent_path()) std::filesystem::create_directories(path.parent_path());
    std::ofstream out(filename, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + filename);
    uint64_t off = 0;
    std::vector<std::pair<const void*, uint64_t>> blocks;
    auto add = [&](const void* ptr, uint64_t bytes) {
      const uint64_t o = off;
      blocks.push_back({ptr, bytes});
      off += 8 + bytes;
      return o;
    };
    const double tv = time;
    const int64_t cv = cycle;
    std::ostringstream x;
    x << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
         "header_type=\"UInt64\">\n<UnstructuredGrid>\n<FieldData>\n";
    x << "<DataArray type=\"Float64\" Name=\"TIME\" NumberOfTuples=\"1\" format=\"appended\" offset=\""
      << add(&tv, 8) << "\"/>\n";
    x << "<DataArray type=\"Int64\" Name=\"CYCLE\" NumberOfTuples=\"1\" format=\"appended\" offset=\"" << add(&cv, 8)
      << "\"/>\n</FieldData>\n";
    x << "<Piece NumberOfPoints=\"" << npts << "\" NumberOfCells=\"" << nsub << "\">\n<Points>\n";
    x << "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"appended\" offset=\""
      << add(pts.data(), pts.size() * 8) << "\"/>\n</Points>\n<Cells>\n";
    x << "<DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\""
      << add(conn.data(), conn.size() * 8) << "\"/>\n";
    x << "<DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"" << add(offs.data(), offs.size() * 8)
      << "\"/>\n";
    x << "<DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"" << add(types.data(), types.size())
      << "\"/>\n</Cells>\n<PointData>\n";
    for (size_t f = 0; f < fields.size(); ++f)
      x << "<DataArray type=\"Float64\" Name=\"" << fields[f].name << "\" NumberOfComponents=\""
        << (fields[f].ncomp > 1 ? 3 : 1) << "\" format=\"appended\" offset=\"" << add(data[f].data(), data[f].size() * 8)
        << "\"/>\n";
    x << "</PointData>\n</Piece>\n</UnstructuredGrid>\n<AppendedData encoding=\"raw\">\n_";
    out << x.str();
    for (auto& [ptr, bytes] : blocks) {
      out.write(reinterpret_cast<const char*>(&bytes), 8);
      out.write(static_cast<const char*>(ptr), (std::streamsize)bytes);
    }
    out << "\n</AppendedData>\n</VTKFile>\n";
    if (!out) throw std::runtime_error("error writing " + filename);
  }

 private:
  Lattice lat;
  const CellList* cl = nullptr;
  unsigned int ns;
  std::vector<double> nodes;
  std::vector<std::vector<double>> I;
};

// parallel record pointing at one piece (write_vtu_with_pvtu_record with one process)
inline void write_pvtu_record(const std::string& pvtu, const std::string& piece, const std::vector<OutputField>& fields) {
  std::ofstream out(pvtu);
  if (!out) throw std::runtime_error("cannot write " + pvtu);
  out << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PUnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
         "header_type=\"UInt64\">\n<PUnstructuredGrid GhostLevel=\"0\">\n<PPointData>\n";
  for (const auto& f : fields)
    out << "<PDataArray type=\"Float64\" Name=\"" << f.name << "\" NumberOfComponents=\"" << (f.ncomp > 1 ? 3 : 1)
        << "\"/>\n";
  out << "</PPointData>\n<PPoints>\n<PDataArray type=\"Float64\" NumberOfComponents=\"3\"/>\n</PPoints>\n";
  out << "<Piece Source=\"" << std::filesystem::path(piece).filename().string() << "\"/>\n</PUnstructuredGrid>\n</VTKFile>\n";
}

}  // namespace output

PRISMS_PF_END_NAMESPACE
