// Exact 64-bit fixed-point arithmetic for the 1-D contractions of the Q1/Q2 cell kernels.
//
// GB300 retires about two FP64 fused multiply-adds per SM per clock, a small fraction of its
// 32-bit integer rate. For Gauss-Lobatto Q1 and Q2 elements the 1-D derivative matrix D[q][j]
// (derivative of basis j at node q on the unit interval) is integral: Q1 {-1, 1}, Q2
// {-3, 4, -1 / -1, 0, 1 / 1, -4, 3}; so are the quadrature weights scaled by 2 (Q1: 1, 1) or 6
// (Q2: 1, 4, 1). The derivative and integration contractions therefore run exactly in 64-bit
// integers, and only their results are rounded back to doubles:
//   * the values being contracted (one cell's nodal values of one component, or one cell's
//     submitted gradient terms of one output component) share a block exponent E, the largest
//     biased IEEE-754 exponent among them;
//   * to_fixed(v, E, top) is v * 2^(1023 + top - E) rounded to an integer (ties away from
//     zero): the largest value of the block lands in [2^top, 2^(top+1)), smaller ones keep
//     every bit down to 2^(E - 1023 - top). The error bound is therefore absolute, relative to
//     the block's largest value: a sum over a line whose own values sit far below the block's
//     largest value keeps that absolute resolution (2^(E - 1023 - top) per term), not 53 bits
//     of its own magnitude. For lines at the block's top exponent this is as fine as the
//     rounding of the FP64 sums it replaces;
//   * integer sums of such values with small integer coefficients are exact while they stay
//     below 2^63 (the callers pick `top` for the headroom of their coefficients);
//   * to_double(x, lsb, sigma) = x * 2^lsb * sigma rounded to nearest, with sigma in [1, 2)
//     held as the 64-bit fraction sigma * 2^63 (the product kept to its integer part); results
//     below the normal range flush to zero and above it become infinities.
// Zeros and subnormal inputs become 0. A block containing an infinity or NaN has E = 2047, and
// its results are quiet NaNs (the finalize kernels then report the non-finite field).
// Written from the IEEE-754 binary64 layout: sign bit 63, biased exponent bits 62..52, 52
// fraction bits with an implicit leading one for normal numbers.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PPF_FX __host__ __device__ __forceinline__
#else
#define PPF_FX inline
#endif

namespace prismspf {
namespace gpu {
namespace fx {

constexpr int EXP_NONFINITE = 2047;
// fixed-point tops of the cell kernels: nodal values below 2^59 leave 3 bits for derivative
// sums (sum |D[q][j]| <= 8); submitted gradient terms below 2^54 leave 9 bits for integration
// sums (sum |iint| <= 8, other-direction weights <= 16, 3 directions)
constexpr int TOP_VALUES = 58;
constexpr int TOP_TERMS = 53;

PPF_FX unsigned long long bits_of(double v) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(v);
#else
  unsigned long long b;
  std::memcpy(&b, &v, 8);
  return b;
#endif
}

PPF_FX double double_of(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double v;
  std::memcpy(&v, &b, 8);
  return v;
#endif
}

PPF_FX int clz64(unsigned long long a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return a ? __builtin_clzll(a) : 64;
#endif
}

PPF_FX unsigned long long mulhi64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

// biased exponent of v (0 for zeros and subnormals, 2047 for infinities and NaNs)
PPF_FX int exponent(double v) { return (int)((bits_of(v) >> 52) & 0x7ff); }

// v * 2^(1023 + top - E) rounded to an integer, ties away from zero; requires exponent(v) <= E
// and 52 <= top <= 60
PPF_FX long long to_fixed(double v, int E, int top) {
  const unsigned long long b = bits_of(v);
  const int e = (int)((b >> 52) & 0x7ff);
  // significand at the top position, then shifted down by E - e with the last bit out rounding
  const unsigned long long m = ((b & 0xfffffffffffffull) | (1ull << 52)) << (top - 52);
#ifdef __CUDA_ARCH__
  const int r = min(E - e, 63);
#else
  const int r = std::min(E - e, 63);
#endif
  unsigned long long a = (m >> r) + (((m << 1) >> r) & 1ull);
  if (e == 0) a = 0;
  const unsigned long long sg = (unsigned long long)((long long)b >> 63);
  return (long long)((a ^ sg) - sg);
}

// x * 2^lsb * sigma, sigma = sig / 2^63 in [1, 2), |x| < 2^63, rounded to nearest (ties to
// even) from floor(|x| * sigma): exact for sigma = 1 and otherwise off by at most half a unit in
// the last place plus 2^lsb, the block's own resolution (the fraction dropped below it)
PPF_FX double to_double(long long x, int lsb, unsigned long long sig) {
  const unsigned long long s = (unsigned long long)x & (1ull << 63);
  const unsigned long long a = x < 0 ? 0ull - (unsigned long long)x : (unsigned long long)x;
  const unsigned long long p = mulhi64(a << 1, sig);  // floor(|x| * sigma)
  const int lz = clz64(p);
  const unsigned long long n = p << (lz & 63);  // leading one at bit 63 (p != 0)
  unsigned long long r = n >> 11;               // 53-bit significand, implicit one at bit 52
  const unsigned int rest = (unsigned int)n & 0x7ffu;
  r += (rest + (unsigned int)(r & 1)) > 0x400u ? 1 : 0;
  const int be = 1086 + lsb - lz;  // biased exponent of n * 2^(lsb - lz)
  if (p == 0 || be <= 0) return double_of(s);
  if (be >= 2047) return double_of(s | 0x7ff0000000000000ull);
  // r carries the implicit one into the exponent field; a rounding carry to 2^53 bumps it
  return double_of(s | (((unsigned long long)(be - 1) << 52) + r));
}

// The lane kernel's conversions (prismspf/gpu/cell_kernel_lanes.cuh). GB300 runs every
// conversion instruction that touches FP64 (int64 <-> double, and float <-> double as well) on
// its FP64 pipe, at the rate of an FP64 fused multiply-add (about two per SM per clock), so these
// are bit operations on 32- and 64-bit integers, written for the shortest instruction sequence
// in the common case: a normal result of a non-zero sum.

// round(v * 2^(1023 + TOP - E)) for exponent(v) <= E, ties away from zero: the same value as
// to_fixed(v, E, TOP) with one variable shift instead of two. 52 <= TOP <= 60.
template <int TOP>
PPF_FX long long to_fixed_fast(double v, int E) {
  static_assert(TOP >= 52 && TOP <= 60, "fixed-point top out of range");
  const unsigned long long b = bits_of(v);
  const int e = (int)((b >> 52) & 0x7ff);
  // significand with one extra bit below it, at the top position
  const unsigned long long m2 = ((b & 0xfffffffffffffull) | (1ull << 52)) << (TOP - 51);
  // (an exponent above E, possible only for the ignored results of a block holding a non-finite
  // value, wraps to a large unsigned shift and clamps like a tiny value)
#ifdef __CUDA_ARCH__
  const unsigned int r = e == 0 ? 63u : min((unsigned int)(E - e), 63u);
#else
  const unsigned int r = e == 0 ? 63u : std::min((unsigned int)(E - e), 63u);
#endif
  const unsigned long long a = ((m2 >> r) + 1) >> 1;
  const unsigned long long sg = (unsigned long long)((long long)b >> 63);
  return (long long)((a ^ sg) - sg);
}

// round(v * sigma * 2^(k + 1023 + TOP - E)) for a scale sigma = sig / 2^63 in [1, 2) and
// exponent(v) + k + 1 <= E, from the floor of the 64-bit product of the significands (off by at
// most half a unit plus 2^-10 units). Zeros and subnormals give 0.
template <int TOP>
PPF_FX long long to_fixed_scaled(double v, int E, unsigned long long sig, int k) {
  static_assert(TOP >= 52 && TOP <= 60, "fixed-point top out of range");
  const unsigned long long b = bits_of(v);
  const int e = (int)((b >> 52) & 0x7ff);
  // P = floor(m * 2^11 * sig / 2^64) in [2^62, 2^64): v * sigma = P * 2^(e - 1085)
  const unsigned long long P = mulhi64(((b & 0xfffffffffffffull) | (1ull << 52)) << 11, sig);
  // (P >> r + 1) >> 1 with r = E - e - k + 61 - TOP >= 2, taken as (P / 2) >> (r - 1) so that
  // the clamped shift stays below 64 for every P
#ifdef __CUDA_ARCH__
  const unsigned int r1 = e == 0 ? 63u : min((unsigned int)(E - e - k + 60 - TOP), 63u);
#else
  const unsigned int r1 = e == 0 ? 63u : std::min((unsigned int)(E - e - k + 60 - TOP), 63u);
#endif
  const unsigned long long a = (((P >> 1) >> r1) + 1) >> 1;
  const unsigned long long sg = (unsigned long long)((long long)b >> 63);
  return (long long)((a ^ sg) - sg);
}

// x * 2^lsb * sigma with sigma = sig / 2^63 in [1, 2) when `scaled` (else 1), |x| < 2^63:
// the product's 64-bit floor (as to_double) rounded to nearest with ties away from zero, which
// differs from to_double's ties-to-even only on exact ties; zero gives +0, results below the
// normal range flush to a signed zero and above it become infinities (as to_double), by selects
// rather than branches.
PPF_FX double to_double_fast(long long x, int lsb, unsigned long long sig, bool scaled) {
  const unsigned long long sg = (unsigned long long)(x >> 63);
  unsigned long long a = ((unsigned long long)x ^ sg) - sg;
  if (scaled) a = mulhi64(a << 1, sig);
  const int lz = clz64(a);  // 64 for a == 0
  const unsigned long long nrm = a << (lz & 63);
  const unsigned long long r = (nrm >> 11) + ((nrm >> 10) & 1ull);  // 53 bits, or 2^53 on a carry
  const int be1 = 1085 + lsb - lz;                                  // biased exponent - 1
  const unsigned long long s63 = sg << 63;
  const unsigned long long bits = s63 | (((unsigned long long)(unsigned int)be1 << 52) + r);
  // zero, below the normal range (signed zero) or above it (signed infinity): the low word is
  // zero and the high word sign (and exponent) only
  const bool ok = (unsigned int)be1 < 2046u && a != 0;
  const unsigned long long edge = a == 0 ? 0ull : (be1 < 0 ? s63 : (s63 | 0x7ff0000000000000ull));
  return double_of(ok ? bits : edge);
}

// Gauss-Lobatto line contractions on the unit interval, exact in integers.
// Derivative at node qd of the line values u: sum_j D[qd][j] u_j with D = {-1, 1 / -1, 1} (Q1)
// or {-3, 4, -1 / -1, 0, 1 / 1, -4, 3} (Q2); for Q2 with a = u2 - u0 and b = 2 (u0 - 2 u1 + u2)
// the three rows are a - b, a, a + b.
template <int n>
PPF_FX long long line_derivative(int qd, long long u0, long long u1, long long u2) {
  if constexpr (n == 2) {
    (void)qd;
    (void)u2;
    return u1 - u0;
  } else {
    const long long a = u2 - u0;
    const long long b = (u0 + u2 - u1 - u1) * 2;
    return qd == 1 ? a : (qd == 0 ? a - b : a + b);
  }
}
// Integration weight of the line terms g at node j: sum_q D[q][j] w(q) g_q with the weights
// times 2 (Q1: 1, 1) or 6 (Q2: 1, 4, 1): Q1 rows -(g0 + g1), g0 + g1; Q2 rows
// {-3, -4, 1 / 4, 0, -4 / -1, 4, 3}, i.e. with A = g2 - g0 and B = g0 + 4 g1 + g2 the rows
// 2A - B, -4A, 2A + B.
template <int n>
PPF_FX long long line_integral(int j, long long g0, long long g1, long long g2) {
  if constexpr (n == 2) {
    (void)g2;
    const long long s = g0 + g1;
    return j == 0 ? -s : s;
  } else {
    const long long A = g2 - g0;
    const long long B = g0 + g2 + g1 * 4;
    return j == 1 ? A * -4 : (j == 0 ? A * 2 - B : A * 2 + B);
  }
}

// n / d for 0 <= n < 2^31 and 1 <= d < 2^31 by a multiply-high (Granlund and Montgomery's
// round-up method): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, q = (hi(n m) + n) >> l
struct FastDiv {
  unsigned int d, m, l;
  PPF_FX void init(unsigned int dd) {
    d = dd;
    l = 0;
    while ((1ull << l) < dd) ++l;
    m = (unsigned int)(((1ull << 32) * ((1ull << l) - dd)) / dd + 1);
  }
  PPF_FX unsigned int div(unsigned int n) const {
#ifdef __CUDA_ARCH__
    return (__umulhi(n, m) + n) >> l;
#else
    return (unsigned int)((((unsigned long long)n * m) >> 32) + n) >> l;
#endif
  }
};

PPF_FX double quiet_nan() { return double_of(0x7ff8000000000000ull); }

// a scale factor s > 0 as s = sigma * 2^k, sigma in [1, 2) held as sigma * 2^63
struct Scale {
  unsigned long long sig;
  int k;
};

inline Scale make_scale(double s) {
  unsigned long long b;
  std::memcpy(&b, &s, 8);
  const int e = (int)((b >> 52) & 0x7ff);
  Scale r;
  r.k = e - 1023;
  r.sig = ((b & 0xfffffffffffffull) | (1ull << 52)) << 11;
  return r;
}

}  // namespace fx
}  // namespace gpu
}  // namespace prismspf
