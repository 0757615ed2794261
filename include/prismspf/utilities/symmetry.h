// Crystal-symmetry anisotropy helpers (reference: include/prismspf/utilities/symmetry.h):
// functions of the angle of an interface normal, for anisotropic gradient-energy
// coefficients such as a(n) = 1 + eps cos(4 theta).
//
//   cos_theta<N>(nx, ny)      cos(N theta), theta the polar angle of the unit normal (nx, ny)
//   sin_theta<N>(nx, ny)      sin(N theta)
//   cos_psi<N>(nx, ny, nz)    cos(N psi), psi the angle of the unit normal from the z axis
//   sin_psi<N>(nx, ny, nz)    sin(N psi)
//   cos_arctan<N>(x)          cos(N atan(x))
//   sin_arctan<N>(x)          sin(N atan(x))
//
// For N <= 5 the multiple-angle values come from Chebyshev polynomials of the unit normal's
// components (cos N t = T_N(cos t), sin N t = sin t U_{N-1}(cos t), by the three-term
// recurrences), which avoids trigonometric calls; larger N use the trigonometric form.
#pragma once

#include <cmath>

#include <prismspf/config.h>
#include <prismspf/dealii_shim.h>

PRISMS_PF_BEGIN_NAMESPACE

namespace Symmetry {

// T_N(c): Chebyshev polynomial of the first kind
template <unsigned int N, typename T>
PPF_HD T chebyshev_t(const T& c) {
  T a = T(1), b = c;
  if (N == 0) return a;
  for (unsigned int k = 1; k < N; ++k) {
    const T next = T(2) * c * b - a;
    a = b;
    b = next;
  }
  return b;
}

// U_N(c): Chebyshev polynomial of the second kind
template <unsigned int N, typename T>
PPF_HD T chebyshev_u(const T& c) {
  T a = T(1), b = T(2) * c;
  if (N == 0) return a;
  for (unsigned int k = 1; k < N; ++k) {
    const T next = T(2) * c * b - a;
    a = b;
    b = next;
  }
  return b;
}

template <unsigned int N, typename T>
PPF_HD T cos_theta(const T& nx, const T& ny) {
  using std::atan2;
  using std::cos;
  if constexpr (N <= 5) {
    (void)ny;
    return chebyshev_t<N>(nx);
  } else {
    return cos(T(N) * atan2(ny, nx));
  }
}

template <unsigned int N, typename T>
PPF_HD T sin_theta(const T& nx, const T& ny) {
  using std::atan2;
  using std::sin;
  if constexpr (N == 0) {
    return T(0);
  } else if constexpr (N <= 5) {
    return ny * chebyshev_u<N - 1>(nx);
  } else {
    return sin(T(N) * atan2(ny, nx));
  }
}

template <unsigned int N, typename T>
PPF_HD T cos_psi(const T& nx, const T& ny, const T& nz) {
  using std::atan2;
  using std::cos;
  using std::sqrt;
  if constexpr (N <= 5) {
    (void)nx;
    (void)ny;
    return chebyshev_t<N>(nz);
  } else {
    return cos(T(N) * atan2(sqrt(nx * nx + ny * ny), nz));
  }
}

template <unsigned int N, typename T>
PPF_HD T sin_psi(const T& nx, const T& ny, const T& nz) {
  using std::atan2;
  using std::sin;
  using std::sqrt;
  const T s = sqrt(nx * nx + ny * ny);
  if constexpr (N == 0) {
    return T(0);
  } else if constexpr (N <= 5) {
    return s * chebyshev_u<N - 1>(nz);
  } else {
    return sin(T(N) * atan2(s, nz));
  }
}

template <unsigned int N, typename T>
PPF_HD T cos_arctan(const T& x) {
  using std::atan;
  using std::cos;
  using std::sqrt;
  if constexpr (N <= 5) {
    return chebyshev_t<N>(T(1) / sqrt(T(1) + x * x));  // cos(atan x) = 1 / sqrt(1 + x^2)
  } else {
    return cos(T(N) * atan(x));
  }
}

template <unsigned int N, typename T>
PPF_HD T sin_arctan(const T& x) {
  using std::atan;
  using std::sin;
  using std::sqrt;
  if constexpr (N == 0) {
    return T(0);
  } else if constexpr (N <= 5) {
    const T c = T(1) / sqrt(T(1) + x * x);
    return x * c * chebyshev_u<N - 1>(c);  // sin(atan x) = x / sqrt(1 + x^2)
  } else {
    return sin(T(N) * atan(x));
  }
}

}  // namespace Symmetry

PRISMS_PF_END_NAMESPACE
