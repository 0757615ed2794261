// Linear elasticity with eigenstrain (applications/mechanics/eshelby_inclusion/custom_pde.h).
// Model constants: 36 Voigt stiffness entries (row-major 6x6; the leading nv x nv block is
// used, nv = 3 in 2-D), e0, width, n_inclusions, then (cx, cy, cz, radius) per inclusion.
// n_inclusions = 0 selects the application's single inclusion of radius 10 at the origin.
// The LHS is compiled in FP64 and FP32 (FP32 for mixed-precision multigrid smoothing).
#include "model_dispatch.cuh"
#include "models.cuh"

namespace ppf {
namespace {

template <int dim, typename number>
size_t make_dim(const double* c, int nc, void* out, size_t cap, std::string* err) {
  using E = Eshelby<dim, 1, number>;  // layout depends on dim and number only
  E o{};
  constexpr int nv = E::nv;
  for (int i = 0; i < nv; ++i)
    for (int j = 0; j < nv; ++j) o.stiffness[i][j] = number(c[i * 6 + j]);
  o.e0 = number(c[36]);
  o.width = number(c[37]);
  o.n_incl = (int)c[38];
  if (o.n_incl < 0 || o.n_incl > ESHELBY_MAX_INCLUSIONS || nc < 39 + 4 * o.n_incl) {
    *err = "eshelby: bad inclusion count or too few constants";
    return 0;
  }
  for (int i = 0; i < o.n_incl; ++i)
    for (int k = 0; k < 4; ++k) o.incl[i][k] = number(c[39 + 4 * i + k]);
  if (sizeof(o) > cap) return 0;
  std::memcpy(out, &o, sizeof(o));
  return sizeof(o);
}

size_t make_object(int dim, int degree, int precision, const double* c, int nc, void* out, size_t cap,
                   std::string* err) {
  (void)degree;
  if (nc < 39) {
    *err = "eshelby expects 36 stiffness entries, e0, width, n_inclusions, inclusions";
    return 0;
  }
  if (dim == 2) return precision ? make_dim<2, float>(c, nc, out, cap, err) : make_dim<2, double>(c, nc, out, cap, err);
  if (dim == 3) return precision ? make_dim<3, float>(c, nc, out, cap, err) : make_dim<3, double>(c, nc, out, cap, err);
  *err = "eshelby: dim must be 2 or 3";
  return 0;
}

const ModelOps ops = {"eshelby", true, make_object, dispatch_launch<Eshelby, true>};
struct Reg {
  Reg() { register_model(&ops); }
} reg;

}  // namespace
}  // namespace ppf
