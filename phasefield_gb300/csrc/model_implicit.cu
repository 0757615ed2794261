// Operator sets of the implicit applications (Newton blocks): "allen_cahn_implicit"
// (Model constants m_well, kappa) and "cahn_hilliard_implicit" (McV, KcV, WcV).
#include "model_dispatch.cuh"
#include "models.cuh"

namespace ppf {
namespace {

template <class O2, class O1>
size_t pack(int precision, const double* c, int ncon, void* out, size_t cap) {
  if (precision == 0) {
    O2 o{};
    double* v = reinterpret_cast<double*>(&o);
    for (int i = 0; i < ncon; ++i) v[i] = c[i];
    if (sizeof(o) > cap) return 0;
    std::memcpy(out, &o, sizeof(o));
    return sizeof(o);
  }
  O1 o{};
  float* v = reinterpret_cast<float*>(&o);
  for (int i = 0; i < ncon; ++i) v[i] = float(c[i]);
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  return sizeof(o);
}

size_t make_ac(int, int, int precision, const double* c, int nc, void* out, size_t cap, std::string* err) {
  if (nc < 2) {
    *err = "allen_cahn_implicit expects Model constants (m_well, kappa)";
    return 0;
  }
  // the object's layout is independent of dim/degree: two numbers
  return pack<AllenCahnImplicit<2, 1, double>, AllenCahnImplicit<2, 1, float>>(precision, c, 2, out, cap);
}

size_t make_ch(int, int, int precision, const double* c, int nc, void* out, size_t cap, std::string* err) {
  if (nc < 3) {
    *err = "cahn_hilliard_implicit expects Model constants (McV, KcV, WcV)";
    return 0;
  }
  return pack<CahnHilliardImplicit<2, 1, double>, CahnHilliardImplicit<2, 1, float>>(precision, c, 3, out, cap);
}

const ModelOps ac_ops = {"allen_cahn_implicit", true, make_ac, dispatch_launch<AllenCahnImplicit, true>};
const ModelOps ch_ops = {"cahn_hilliard_implicit", true, make_ch, dispatch_launch<CahnHilliardImplicit, true>};
struct Reg {
  Reg() {
    register_model(&ac_ops);
    register_model(&ch_ops);
  }
} reg;

}  // namespace
}  // namespace ppf
