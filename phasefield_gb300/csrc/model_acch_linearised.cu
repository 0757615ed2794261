// Tangent-linear and adjoint operator sets of the coupled Allen-Cahn / Cahn-Hilliard explicit
// block (constants Mc, Mn, Kn; the tangent also takes the parameter direction dMc, dKn).
#include "model_dispatch.cuh"
#include "models.cuh"

namespace ppf {
namespace {

size_t make_tangent(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                    std::string* err) {
  (void)dim;
  (void)degree;
  if (precision != 0 || nc < 5) {
    *err = "coupled_acch_tangent expects (Mc, Mn, Kn, dMc, dKn), FP64";
    return 0;
  }
  CoupledACCHTangent<2, 1, double> o{c[0], c[1], c[2], c[3], c[4]};
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  return sizeof(o);
}

size_t make_adjoint(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                    std::string* err) {
  (void)dim;
  (void)degree;
  if (precision != 0 || nc < 3) {
    *err = "coupled_acch_adjoint expects (Mc, Mn, Kn), FP64";
    return 0;
  }
  CoupledACCHAdjoint<2, 1, double> o{c[0], c[1], c[2]};
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  return sizeof(o);
}

const ModelOps tangent_ops = {"coupled_acch_tangent", false, make_tangent, dispatch_launch<CoupledACCHTangent, false>};
const ModelOps adjoint_ops = {"coupled_acch_adjoint", false, make_adjoint, dispatch_launch<CoupledACCHAdjoint, false>};
struct Reg {
  Reg() {
    register_model(&tangent_ops);
    register_model(&adjoint_ops);
  }
} reg;

}  // namespace
}  // namespace ppf
