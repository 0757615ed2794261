// Minimal device-capable stand-ins for the deal.II value types that PRISMS-PF user
// callbacks use: VectorizedArray, Tensor<1|2|3>, SymmetricTensor<2>, Point.
//
// The reference callbacks (e.g. applications/allen_cahn/explicit/custom_pde.h:72-101)
// manipulate `dealii::VectorizedArray<number>` lanes and `dealii::Tensor<rank,dim,...>`.
// On the GPU one thread owns one quadrature point, so VectorizedArray is a width-1 wrapper
// and every operation is __host__ __device__. Only the operations the PRISMS-PF callbacks
// use are provided; names and semantics follow deal.II (Tensor<1>*Tensor<1> is the scalar
// product, Tensor<2>*Tensor<1> contracts the last index).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define PPF_HD __host__ __device__ __forceinline__
#else
#define PPF_HD inline
#endif

namespace dealii {

template <typename Number>
struct VectorizedArray {
  using value_type = Number;
  Number v;
  PPF_HD VectorizedArray() : v(0) {}
  PPF_HD VectorizedArray(Number x) : v(x) {}
  template <typename T, typename = decltype(Number(T()))>
  PPF_HD VectorizedArray(T x) : v(Number(x)) {}
  static constexpr unsigned int size() { return 1; }
  PPF_HD Number& operator[](unsigned int) { return v; }
  PPF_HD const Number& operator[](unsigned int) const { return v; }
  PPF_HD VectorizedArray& operator+=(const VectorizedArray& o) { v += o.v; return *this; }
  PPF_HD VectorizedArray& operator-=(const VectorizedArray& o) { v -= o.v; return *this; }
  PPF_HD VectorizedArray& operator*=(const VectorizedArray& o) { v *= o.v; return *this; }
  PPF_HD VectorizedArray& operator/=(const VectorizedArray& o) { v /= o.v; return *this; }
  PPF_HD VectorizedArray& operator=(Number x) { v = x; return *this; }
  PPF_HD operator Number() const { return v; }
};

template <typename N> PPF_HD VectorizedArray<N> operator+(VectorizedArray<N> a, VectorizedArray<N> b) { return a.v + b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator-(VectorizedArray<N> a, VectorizedArray<N> b) { return a.v - b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator*(VectorizedArray<N> a, VectorizedArray<N> b) { return a.v * b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator/(VectorizedArray<N> a, VectorizedArray<N> b) { return a.v / b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator-(VectorizedArray<N> a) { return -a.v; }
template <typename N> PPF_HD VectorizedArray<N> operator+(VectorizedArray<N> a, N b) { return a.v + b; }
template <typename N> PPF_HD VectorizedArray<N> operator+(N a, VectorizedArray<N> b) { return a + b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator-(VectorizedArray<N> a, N b) { return a.v - b; }
template <typename N> PPF_HD VectorizedArray<N> operator-(N a, VectorizedArray<N> b) { return a - b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator*(VectorizedArray<N> a, N b) { return a.v * b; }
template <typename N> PPF_HD VectorizedArray<N> operator*(N a, VectorizedArray<N> b) { return a * b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator/(VectorizedArray<N> a, N b) { return a.v / b; }
template <typename N> PPF_HD VectorizedArray<N> operator/(N a, VectorizedArray<N> b) { return a / b.v; }
// integer literals (e.g. `2 * a2 * c`) promote to Number
template <typename N> PPF_HD VectorizedArray<N> operator*(int a, VectorizedArray<N> b) { return N(a) * b.v; }
template <typename N> PPF_HD VectorizedArray<N> operator*(VectorizedArray<N> a, int b) { return a.v * N(b); }
// double literals with single-precision lanes (as deal.II's VectorizedArray<float> accepts)
PPF_HD VectorizedArray<float> operator+(VectorizedArray<float> a, double b) { return a.v + float(b); }
PPF_HD VectorizedArray<float> operator+(double a, VectorizedArray<float> b) { return float(a) + b.v; }
PPF_HD VectorizedArray<float> operator-(VectorizedArray<float> a, double b) { return a.v - float(b); }
PPF_HD VectorizedArray<float> operator-(double a, VectorizedArray<float> b) { return float(a) - b.v; }
PPF_HD VectorizedArray<float> operator*(VectorizedArray<float> a, double b) { return a.v * float(b); }
PPF_HD VectorizedArray<float> operator*(double a, VectorizedArray<float> b) { return float(a) * b.v; }
PPF_HD VectorizedArray<float> operator/(VectorizedArray<float> a, double b) { return a.v / float(b); }
PPF_HD VectorizedArray<float> operator/(double a, VectorizedArray<float> b) { return float(a) / b.v; }

template <typename Number>
PPF_HD VectorizedArray<Number> make_vectorized_array(Number x) { return VectorizedArray<Number>(x); }

// ----------------------------------------------------------------------------------------
// Tensor<rank, dim, T>
// ----------------------------------------------------------------------------------------
template <int rank, int dim, typename T = double>
struct Tensor;

template <int dim, typename T>
struct Tensor<0, dim, T> {
  // rank-0 tensors decay to their scalar in deal.II; mirrored for completeness
  T value{};
};

template <int dim, typename T>
struct Tensor<1, dim, T> {
  static constexpr unsigned int rank = 1;
  static constexpr unsigned int dimension = dim;
  static constexpr unsigned int n_independent_components = dim;
  T values[dim];
  PPF_HD Tensor() { for (int i = 0; i < dim; ++i) values[i] = T(0.0); }
  // from an array of components, e.g. Tensor<1, 2>({200.0, 200.0})
  PPF_HD explicit Tensor(const T (&init)[dim]) { for (int i = 0; i < dim; ++i) values[i] = init[i]; }
  PPF_HD T& operator[](unsigned int i) { return values[i]; }
  PPF_HD const T& operator[](unsigned int i) const { return values[i]; }
  PPF_HD Tensor& operator+=(const Tensor& o) { for (int i = 0; i < dim; ++i) values[i] += o.values[i]; return *this; }
  PPF_HD Tensor& operator-=(const Tensor& o) { for (int i = 0; i < dim; ++i) values[i] -= o.values[i]; return *this; }
  template <typename S> PPF_HD Tensor& operator*=(const S& s) { for (int i = 0; i < dim; ++i) values[i] = values[i] * s; return *this; }
  template <typename S> PPF_HD Tensor& operator/=(const S& s) { for (int i = 0; i < dim; ++i) values[i] = values[i] / s; return *this; }
  PPF_HD T norm_square() const { T s = values[0] * values[0]; for (int i = 1; i < dim; ++i) s = s + values[i] * values[i]; return s; }
  PPF_HD T norm() const;
  PPF_HD void clear() { for (int i = 0; i < dim; ++i) values[i] = T(0.0); }
};

template <int dim, typename T>
struct Tensor<2, dim, T> {
  static constexpr unsigned int rank = 2;
  static constexpr unsigned int dimension = dim;
  static constexpr unsigned int n_independent_components = dim * dim;
  Tensor<1, dim, T> values[dim];
  PPF_HD Tensor() {}
  PPF_HD Tensor<1, dim, T>& operator[](unsigned int i) { return values[i]; }
  PPF_HD const Tensor<1, dim, T>& operator[](unsigned int i) const { return values[i]; }
  PPF_HD Tensor& operator+=(const Tensor& o) { for (int i = 0; i < dim; ++i) values[i] += o.values[i]; return *this; }
  PPF_HD Tensor& operator-=(const Tensor& o) { for (int i = 0; i < dim; ++i) values[i] -= o.values[i]; return *this; }
  template <typename S> PPF_HD Tensor& operator*=(const S& s) { for (int i = 0; i < dim; ++i) values[i] *= s; return *this; }
  PPF_HD T norm_square() const { T s = values[0].norm_square(); for (int i = 1; i < dim; ++i) s = s + values[i].norm_square(); return s; }
  PPF_HD T norm() const;
  PPF_HD void clear() { for (int i = 0; i < dim; ++i) values[i].clear(); }
};

template <int dim, typename T>
struct Tensor<3, dim, T> {
  static constexpr unsigned int rank = 3;
  static constexpr unsigned int dimension = dim;
  Tensor<2, dim, T> values[dim];
  PPF_HD Tensor() {}
  PPF_HD Tensor<2, dim, T>& operator[](unsigned int i) { return values[i]; }
  PPF_HD const Tensor<2, dim, T>& operator[](unsigned int i) const { return values[i]; }
};

}  // namespace dealii

// math on the width-1 VectorizedArray (deal.II provides these overloads in std as well)
namespace std {
template <typename N> PPF_HD dealii::VectorizedArray<N> sqrt(dealii::VectorizedArray<N> x) { return ::sqrt(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> tanh(dealii::VectorizedArray<N> x) { return ::tanh(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> exp(dealii::VectorizedArray<N> x) { return ::exp(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> log(dealii::VectorizedArray<N> x) { return ::log(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> sin(dealii::VectorizedArray<N> x) { return ::sin(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> cos(dealii::VectorizedArray<N> x) { return ::cos(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> abs(dealii::VectorizedArray<N> x) { return ::fabs(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> pow(dealii::VectorizedArray<N> x, N p) { return ::pow(x.v, p); }
template <typename N> PPF_HD dealii::VectorizedArray<N> pow(dealii::VectorizedArray<N> x, dealii::VectorizedArray<N> p) { return ::pow(x.v, p.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> min(dealii::VectorizedArray<N> a, dealii::VectorizedArray<N> b) { return a.v < b.v ? a.v : b.v; }
template <typename N> PPF_HD dealii::VectorizedArray<N> max(dealii::VectorizedArray<N> a, dealii::VectorizedArray<N> b) { return a.v > b.v ? a.v : b.v; }
template <typename N> PPF_HD dealii::VectorizedArray<N> atan(dealii::VectorizedArray<N> x) { return ::atan(x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> atan2(dealii::VectorizedArray<N> y, dealii::VectorizedArray<N> x) { return ::atan2(y.v, x.v); }
template <typename N> PPF_HD dealii::VectorizedArray<N> erf(dealii::VectorizedArray<N> x) { return ::erf(x.v); }
}  // namespace std

namespace dealii {

template <int dim, typename T> PPF_HD T Tensor<1, dim, T>::norm() const { using std::sqrt; return sqrt(norm_square()); }
template <int dim, typename T> PPF_HD T Tensor<2, dim, T>::norm() const { using std::sqrt; return sqrt(norm_square()); }

// rank-1 arithmetic
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator+(Tensor<1, dim, T> a, const Tensor<1, dim, T>& b) { a += b; return a; }
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator-(Tensor<1, dim, T> a, const Tensor<1, dim, T>& b) { a -= b; return a; }
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator-(Tensor<1, dim, T> a) { for (int i = 0; i < dim; ++i) a.values[i] = -a.values[i]; return a; }
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator*(Tensor<1, dim, T> a, const T& s) { for (int i = 0; i < dim; ++i) a.values[i] = a.values[i] * s; return a; }
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator*(const T& s, Tensor<1, dim, T> a) { for (int i = 0; i < dim; ++i) a.values[i] = s * a.values[i]; return a; }
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator/(Tensor<1, dim, T> a, const T& s) { for (int i = 0; i < dim; ++i) a.values[i] = a.values[i] / s; return a; }
template <int dim, typename N> PPF_HD Tensor<1, dim, VectorizedArray<N>> operator*(Tensor<1, dim, VectorizedArray<N>> a, N s) { for (int i = 0; i < dim; ++i) a.values[i] = a.values[i] * s; return a; }
template <int dim, typename N> PPF_HD Tensor<1, dim, VectorizedArray<N>> operator*(N s, Tensor<1, dim, VectorizedArray<N>> a) { for (int i = 0; i < dim; ++i) a.values[i] = s * a.values[i]; return a; }
template <int dim, typename N> PPF_HD Tensor<1, dim, VectorizedArray<N>> operator/(Tensor<1, dim, VectorizedArray<N>> a, N s) { for (int i = 0; i < dim; ++i) a.values[i] = a.values[i] / s; return a; }
// scalar product
template <int dim, typename T> PPF_HD T operator*(const Tensor<1, dim, T>& a, const Tensor<1, dim, T>& b) { T s = a.values[0] * b.values[0]; for (int i = 1; i < dim; ++i) s = s + a.values[i] * b.values[i]; return s; }
template <int dim, typename T> PPF_HD T scalar_product(const Tensor<1, dim, T>& a, const Tensor<1, dim, T>& b) { return a * b; }

// rank-2 arithmetic
template <int dim, typename T> PPF_HD Tensor<2, dim, T> operator+(Tensor<2, dim, T> a, const Tensor<2, dim, T>& b) { a += b; return a; }
template <int dim, typename T> PPF_HD Tensor<2, dim, T> operator-(Tensor<2, dim, T> a, const Tensor<2, dim, T>& b) { a -= b; return a; }
template <int dim, typename T> PPF_HD Tensor<2, dim, T> operator-(Tensor<2, dim, T> a) { for (int i = 0; i < dim; ++i) a.values[i] = -a.values[i]; return a; }
template <int dim, typename T> PPF_HD Tensor<2, dim, T> operator*(Tensor<2, dim, T> a, const T& s) { for (int i = 0; i < dim; ++i) a.values[i] = a.values[i] * s; return a; }
template <int dim, typename T> PPF_HD Tensor<2, dim, T> operator*(const T& s, Tensor<2, dim, T> a) { for (int i = 0; i < dim; ++i) a.values[i] = s * a.values[i]; return a; }
template <int dim, typename N> PPF_HD Tensor<2, dim, VectorizedArray<N>> operator*(Tensor<2, dim, VectorizedArray<N>> a, N s) { for (int i = 0; i < dim; ++i) a.values[i] = a.values[i] * s; return a; }
template <int dim, typename N> PPF_HD Tensor<2, dim, VectorizedArray<N>> operator*(N s, Tensor<2, dim, VectorizedArray<N>> a) { for (int i = 0; i < dim; ++i) a.values[i] = s * a.values[i]; return a; }
// contraction of the last index
template <int dim, typename T> PPF_HD Tensor<1, dim, T> operator*(const Tensor<2, dim, T>& A, const Tensor<1, dim, T>& x) { Tensor<1, dim, T> y; for (int i = 0; i < dim; ++i) y.values[i] = A.values[i] * x; return y; }
template <int dim, typename T> PPF_HD Tensor<2, dim, T> operator*(const Tensor<2, dim, T>& A, const Tensor<2, dim, T>& B) {
  Tensor<2, dim, T> C;
  for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) { T s = A[i][0] * B[0][j]; for (int k = 1; k < dim; ++k) s = s + A[i][k] * B[k][j]; C[i][j] = s; }
  return C;
}
template <int dim, typename T> PPF_HD T trace(const Tensor<2, dim, T>& A) { T s = A[0][0]; for (int i = 1; i < dim; ++i) s = s + A[i][i]; return s; }
template <int dim, typename T> PPF_HD Tensor<2, dim, T> transpose(const Tensor<2, dim, T>& A) { Tensor<2, dim, T> B; for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) B[i][j] = A[j][i]; return B; }
template <int dim, typename T> PPF_HD T scalar_product(const Tensor<2, dim, T>& a, const Tensor<2, dim, T>& b) { T s = a[0] * b[0]; for (int i = 1; i < dim; ++i) s = s + a[i] * b[i]; return s; }
template <int dim, typename T> PPF_HD T double_contract(const Tensor<2, dim, T>& a, const Tensor<2, dim, T>& b) { return scalar_product(a, b); }

// Tensor<2, n, Number> * Tensor<1, n, VectorizedArray<Number>> (elasticity matrix times Voigt vector)
template <int n, typename N>
PPF_HD Tensor<1, n, VectorizedArray<N>> operator*(const Tensor<2, n, N>& A, const Tensor<1, n, VectorizedArray<N>>& x) {
  Tensor<1, n, VectorizedArray<N>> y;
  for (int i = 0; i < n; ++i) { VectorizedArray<N> s = A[i][0] * x[0]; for (int j = 1; j < n; ++j) s = s + A[i][j] * x[j]; y[i] = s; }
  return y;
}

// ----------------------------------------------------------------------------------------
// SymmetricTensor<2, dim, T>: stored as a full tensor with symmetric entries.
// ----------------------------------------------------------------------------------------
template <int rank, int dim, typename T = double>
struct SymmetricTensor;

template <int dim, typename T>
struct SymmetricTensor<2, dim, T> {
  static constexpr unsigned int rank = 2;
  T a[dim][dim];
  PPF_HD SymmetricTensor() { for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) a[i][j] = T(0.0); }
  PPF_HD T operator()(unsigned int i, unsigned int j) const { return a[i][j]; }
  PPF_HD T& operator()(unsigned int i, unsigned int j) { return a[i][j]; }
  struct Row { T* r; PPF_HD T& operator[](unsigned int j) { return r[j]; } };
  struct CRow { const T* r; PPF_HD const T& operator[](unsigned int j) const { return r[j]; } };
  PPF_HD Row operator[](unsigned int i) { return Row{a[i]}; }
  PPF_HD CRow operator[](unsigned int i) const { return CRow{a[i]}; }
  PPF_HD operator Tensor<2, dim, T>() const { Tensor<2, dim, T> t; for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) t[i][j] = a[i][j]; return t; }
  PPF_HD T norm() const { using std::sqrt; T s = a[0][0] * a[0][0]; for (int i = 0; i < dim; ++i) for (int j = 0; j < dim; ++j) if (i || j) s = s + a[i][j] * a[i][j]; return sqrt(s); }
};
template <int dim, typename T> PPF_HD T trace(const SymmetricTensor<2, dim, T>& A) { T s = A.a[0][0]; for (int i = 1; i < dim; ++i) s = s + A.a[i][i]; return s; }

// ----------------------------------------------------------------------------------------
// Point<dim, T>
// ----------------------------------------------------------------------------------------
template <int dim, typename T = double>
struct Point : public Tensor<1, dim, T> {
  PPF_HD Point() {}
  PPF_HD Point(const Tensor<1, dim, T>& t) : Tensor<1, dim, T>(t) {}
  PPF_HD Point(T x, T y) { this->values[0] = x; if (dim > 1) this->values[1] = y; }
  PPF_HD Point(T x, T y, T z) { this->values[0] = x; if (dim > 1) this->values[1] = y; if (dim > 2) this->values[2] = z; }
  PPF_HD T distance(const Point& o) const { return (Tensor<1, dim, T>(*this) - Tensor<1, dim, T>(o)).norm(); }
};

// ----------------------------------------------------------------------------------------
// EvaluationFlags (the dependency flags of a solve block; host side)
// ----------------------------------------------------------------------------------------
namespace EvaluationFlags {
enum EvaluationFlags { nothing = 0, values = 1, gradients = 2, hessians = 4 };
inline constexpr EvaluationFlags operator|(EvaluationFlags a, EvaluationFlags b) {
  return static_cast<EvaluationFlags>(static_cast<int>(a) | static_cast<int>(b));
}
inline constexpr EvaluationFlags operator&(EvaluationFlags a, EvaluationFlags b) {
  return static_cast<EvaluationFlags>(static_cast<int>(a) & static_cast<int>(b));
}
inline EvaluationFlags& operator|=(EvaluationFlags& a, EvaluationFlags b) { return a = a | b; }
inline EvaluationFlags& operator&=(EvaluationFlags& a, EvaluationFlags b) { return a = a & b; }
}  // namespace EvaluationFlags

}  // namespace dealii
