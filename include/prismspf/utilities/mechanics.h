// Voigt-notation stress helper with the interface of the reference's
// include/prismspf/utilities/mechanics.h:18-109 (compute_stress from a Voigt strain or from
// a rank-2 strain; shear strains enter as engineering strains).
#pragma once

#include <prismspf/config.h>
#include <prismspf/dealii_shim.h>

PRISMS_PF_BEGIN_NAMESPACE

namespace Mechanics {

template <unsigned int dim>
constexpr unsigned int voigt_tensor_size = (2 * dim) - 1 + (dim / 3);

template <unsigned int dim, typename T, typename C>
PPF_HD void compute_stress(const dealii::Tensor<2, voigt_tensor_size<dim>, C>& elasticity_tensor,
                           const dealii::Tensor<1, voigt_tensor_size<dim>, T>& strain,
                           dealii::Tensor<1, voigt_tensor_size<dim>, T>& stress) {
  constexpr int nv = voigt_tensor_size<dim>;
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
