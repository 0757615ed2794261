// Voigt-notation stress helper with the interface of the reference's
// include/prismspf/utilities/mechanics.h:18-109 (compute_stress from a Voigt strain or from
// a rank-2 strain; shear strains enter as engineering strains).
#pragma once

#include <prismspf/config.h>
#include <prismspf/dealii_shim.h>

#include <type_traits>

PRISMS_PF_BEGIN_NAMESPACE

namespace Mechanics {

template <unsigned int dim>
constexpr unsigned int voigt_tensor_size = (2 * dim) - 1 + (dim / 3);

namespace detail {
// +0 or -0, tested on the bits (an integer test: on GB300 a floating-point compare of doubles
// runs on the narrow FP64 pipe)
PPF_HD bool zero_bits(double c) {
#ifdef __CUDA_ARCH__
  return ((unsigned long long)__double_as_longlong(c) << 1) == 0ull;
#else
  return c == 0.0;
#endif
}
PPF_HD bool zero_bits(float c) {
#ifdef __CUDA_ARCH__
  return ((unsigned int)__float_as_int(c) << 1) == 0u;
#else
  return c == 0.0f;
#endif
}
template <typename C>
PPF_HD bool stiffness_zero(const C& c) {
  if constexpr (std::is_arithmetic<C>::value) return zero_bits(c);
  else return zero_bits(c.v);
}
// whether a Voigt stiffness couples normal and shear strains nowhere and each shear strain only
// to its own stress (orthotropic axes along the mesh: cubic and isotropic materials included)
template <int nv, typename C>
PPF_HD bool orthotropic(const dealii::Tensor<2, nv, C>& c) {
  constexpr int nn = nv == 6 ? 3 : (nv == 3 ? 2 : 1);  // normal components
  bool z = true;
  for (int i = 0; i < nv; ++i)
    for (int j = 0; j < nv; ++j)
      if ((i < nn) != (j < nn) || (i >= nn && j != i)) z = z && stiffness_zero(c[i][j]);
  return z;
}
}  // namespace detail

// sigma = C epsilon (Voigt). An orthotropic stiffness (see detail::orthotropic) takes the
// products of its non-zero blocks only: 12 of the 36 multiply-adds in 3-D, the same sums in the
// same order as the dense product less its terms with an exactly zero coefficient (equal for
// finite strains up to the sign of an exact zero). The stiffness is the same at every point of a
// launch (a kernel parameter), so on the GPU the test is uniform and leaves the point loop.
template <unsigned int dim, typename T, typename C>
PPF_HD void compute_stress(const dealii::Tensor<2, voigt_tensor_size<dim>, C>& elasticity_tensor,
                           const dealii::Tensor<1, voigt_tensor_size<dim>, T>& strain,
                           dealii::Tensor<1, voigt_tensor_size<dim>, T>& stress) {
  constexpr int nv = voigt_tensor_size<dim>;
  constexpr int nn = nv == 6 ? 3 : (nv == 3 ? 2 : 1);
  if (detail::orthotropic<nv, C>(elasticity_tensor)) {
    for (int i = 0; i < nn; ++i) {
      T s = elasticity_tensor[i][0] * strain[0];
      for (int j = 1; j < nn; ++j) s = s + elasticity_tensor[i][j] * strain[j];
      stress[i] = s;
    }
    for (int i = nn; i < nv; ++i) stress[i] = elasticity_tensor[i][i] * strain[i];
    return;
  }
  for (int i = 0; i < nv; ++i) {
    T s = elasticity_tensor[i][0] * strain[0];
    for (int j = 1; j < nv; ++j) s = s + elasticity_tensor[i][j] * strain[j];
    stress[i] = s;
  }
}

template <unsigned int dim, typename T, typename C>
PPF_HD void compute_stress(const dealii::Tensor<2, voigt_tensor_size<dim>, C>& elasticity_tensor,
                           const dealii::Tensor<2, dim, T>& strain,
                           dealii::Tensor<2, dim, T>& stress) {
  constexpr int nv = voigt_tensor_size<dim>;
  dealii::Tensor<1, nv, T> eps, sig;
  if constexpr (dim == 3) {
    eps[0] = strain[0][0];
    eps[1] = strain[1][1];
    eps[2] = strain[2][2];
    eps[3] = strain[1][2] + strain[2][1];
    eps[4] = strain[0][2] + strain[2][0];
    eps[5] = strain[0][1] + strain[1][0];
    compute_stress<dim, T, C>(elasticity_tensor, eps, sig);
    stress[0][0] = sig[0];
    stress[1][1] = sig[1];
    stress[2][2] = sig[2];
    stress[1][2] = sig[3];
    stress[2][1] = sig[3];
    stress[0][2] = sig[4];
    stress[2][0] = sig[4];
    stress[0][1] = sig[5];
    stress[1][0] = sig[5];
  } else if constexpr (dim == 2) {
    eps[0] = strain[0][0];
    eps[1] = strain[1][1];
    eps[2] = strain[0][1] + strain[1][0];
    compute_stress<dim, T, C>(elasticity_tensor, eps, sig);
    stress[0][0] = sig[0];
    stress[1][1] = sig[1];
    stress[0][1] = sig[2];
    stress[1][0] = sig[2];
  } else {
    stress[0][0] = elasticity_tensor[0][0] * strain[0][0];
  }
}

}  // namespace Mechanics

PRISMS_PF_END_NAMESPACE
