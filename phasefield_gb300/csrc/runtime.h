// Internal host runtime of the GB300 engine (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include <prismspf/gpu/cell_kernel.cuh>

namespace ppf {

// A compiled PDE operator set (one user CustomPDE): how to build its device object from the
// Model constants and how to launch its cell kernel for a (dim, degree, mode, precision).
struct ModelOps {
  const char* name;
  bool has_lhs;
  // fills `out` (capacity `cap` bytes) with the device object in the given precision
  // (0 FP64, 1 FP32); returns its size, 0 on error
  size_t (*make_object)(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                        std::string* err);
  // launches cell_kernel<PDE, dim, degree, mode, number>
  cudaError_t (*launch)(int dim, int degree, int mode, int precision, const CellLaunch& P, const void* obj,
                        size_t smem, cudaStream_t s);
};

const ModelOps* find_model(const char* name);
void register_model(const ModelOps* ops);

// threads per block of the cell kernel for (dim, degree)
int cell_threads(int dim, int degree);
size_t cell_smem(int dim, int degree, int precision, int nrows_in, int nrows_out);
// builds CellTables<dim,degree,number> bytes (precision 0 FP64, 1 FP32)
// fx_rows: value rows the FP64 Q1/Q2 kernels keep a fixed-point copy of (rows read as gradients);
// val_rows: value rows the lane kernel keeps a double copy of (rows read as values or Hessians)
std::vector<unsigned char> build_cell_tables(int dim, int degree, int precision, const double* lo, const double* h,
                                             const signed char slot_of[pg::MAX_FIELDS][pg::NAGE],
                                             const signed char* slot_comp0, const signed char* out_of,
                                             const signed char* out_row0, unsigned int fx_rows = 0xffffffffu,
                                             unsigned int val_rows = 0xffffffffu);
// whether FP64 tables allow the lane kernel (integer contractions, cubic cells)
bool tables_lanes(const std::vector<unsigned char>& tab, int dim, int degree);
// the launch-record fields of contraction mode m (1-4)
void set_fx_mode(CellLaunch& L, int m);
// PPF_CONTRACTION_MODE (1-4, mode 4 only where the lane kernel applies, else 1), 0 when unset
int env_fx_mode(bool lanes_ok);

}  // namespace ppf
