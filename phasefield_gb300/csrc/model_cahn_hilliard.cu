// Cahn-Hilliard operator set (applications/cahn_hilliard/explicit/custom_pde.h).
// Model constants: McV, KcV, WcV.
#include "model_dispatch.cuh"
#include "models.cuh"

namespace ppf {
namespace {

size_t make_object(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                   std::string* err) {
  if (precision != 0) {
    *err = "cahn_hilliard: only the FP64 operator is compiled";
    return 0;
  }
  if (nc < 3) {
    *err = "cahn_hilliard expects Model constants (McV, KcV, WcV)";
    return 0;
  }
  CahnHilliard<2, 1, double> o{c[0], c[1], c[2]};  // layout is independent of dim/degree
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  (void)dim;
  (void)degree;
  return sizeof(o);
}

const ModelOps ops = {"cahn_hilliard", false, make_object, dispatch_launch<CahnHilliard, false>};
struct Reg {
  Reg() { register_model(&ops); }
} reg;

}  // namespace
}  // namespace ppf
