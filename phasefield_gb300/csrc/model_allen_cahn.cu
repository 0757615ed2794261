// Allen-Cahn operator set (applications/allen_cahn/explicit/custom_pde.h).
// Model constants: m_well, kappa.
#include "model_dispatch.cuh"
#include "models.cuh"

namespace ppf {
namespace {

size_t make_object(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                   std::string* err) {
  if (precision != 0) {
    *err = "allen_cahn: only the FP64 operator is compiled";
    return 0;
  }
  if (nc < 2) {
    *err = "allen_cahn expects Model constants (m_well, kappa)";
    return 0;
  }
  AllenCahn<2, 1, double> o{c[0], c[1]};  // layout is independent of dim/degree
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  (void)dim;
  (void)degree;
  return sizeof(o);
}

const ModelOps ops = {"allen_cahn", false, make_object, dispatch_launch<AllenCahn, false>};
struct Reg {
  Reg() { register_model(&ops); }
} reg;

}  // namespace
}  // namespace ppf
