// Coupled Allen-Cahn / Cahn-Hilliard operator set
// (applications/coupled_allen_cahn_cahn_hilliard/custom_pde.h). Model constants: Mc, Mn, Kn.
#include "model_dispatch.cuh"
#include "models.cuh"

namespace ppf {
namespace {

size_t make_object(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                   std::string* err) {
  if (precision != 0) {
    *err = "coupled_acch: only the FP64 operator is compiled";
    return 0;
  }
  if (nc < 3) {
    *err = "coupled_acch expects Model constants (Mc, Mn, Kn)";
    return 0;
  }
  CoupledACCH<2, 1, double> o{c[0], c[1], c[2]};  // layout is independent of dim/degree
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  (void)dim;
  (void)degree;
  return sizeof(o);
}

const ModelOps ops = {"coupled_acch", false, make_object, dispatch_launch<CoupledACCH, false>};
struct Reg {
  Reg() { register_model(&ops); }
} reg;

}  // namespace
}  // namespace ppf
