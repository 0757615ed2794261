// C entry points over include/prismspf/gpu/fixed_point.cuh for the host tests of the
// fixed-point conversions (compiled with g++ by tests/test_fixed_point_host.py).
#include <prismspf/gpu/fixed_point.cuh>

namespace fx = prismspf::gpu::fx;

extern "C" {
int fxs_exponent(double v) { return fx::exponent(v); }
long long fxs_to_fixed(double v, int E, int top) { return fx::to_fixed(v, E, top); }
double fxs_to_double(long long x, int lsb, unsigned long long sig) { return fx::to_double(x, lsb, sig); }
void fxs_make_scale(double s, unsigned long long* sig, int* k) {
  const fx::Scale r = fx::make_scale(s);
  *sig = r.sig;
  *k = r.k;
}
unsigned int fxs_fastdiv(unsigned int n, unsigned int d) {
  fx::FastDiv f;
  f.init(d);
  return f.div(n);
}
long long fxs_to_fixed_fast(double v, int E, int top) {
  switch (top) {
    case 52: return fx::to_fixed_fast<52>(v, E);
    case 53: return fx::to_fixed_fast<53>(v, E);
    case 58: return fx::to_fixed_fast<58>(v, E);
    default: return fx::to_fixed_fast<60>(v, E);
  }
}
long long fxs_to_fixed_scaled(double v, int E, unsigned long long sig, int k) {
  return fx::to_fixed_scaled<52>(v, E, sig, k);
}
double fxs_to_double_fast(long long x, int lsb, unsigned long long sig, int scaled) {
  return fx::to_double_fast(x, lsb, sig, scaled != 0);
}
long long fxs_line_derivative(int n, int qd, long long u0, long long u1, long long u2) {
  return n == 2 ? fx::line_derivative<2>(qd, u0, u1, u2) : fx::line_derivative<3>(qd, u0, u1, u2);
}
long long fxs_line_integral(int n, int j, long long g0, long long g1, long long g2) {
  return n == 2 ? fx::line_integral<2>(j, g0, g1, g2) : fx::line_integral<3>(j, g0, g1, g2);
}
void fxs_to_fixed_n(const double* v, long long n, int E, int top, long long* out) {
  for (long long i = 0; i < n; ++i) out[i] = fx::to_fixed(v[i], E, top);
}
void fxs_to_double_n(const long long* x, long long n, int lsb, unsigned long long sig, double* out) {
  for (long long i = 0; i < n; ++i) out[i] = fx::to_double(x[i], lsb, sig);
}
}
